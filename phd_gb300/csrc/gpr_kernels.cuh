// gpr_kernels.cuh - the ADER-WENO step kernels (N = 2), templated on the
// variable layout (THERMAL, LSET).  Host-side launchers live in gpr_capi.cu.
#pragma once

#include "gpr_consts.cuh"
#include "gpr_device.cuh"

namespace gpr {

constexpr double LAMS = 1.0;       // WENO side-stencil weight (options.h:24)
constexpr double WENO_EPS = 1e-14; // options.h:26

template <bool TH, int LS> struct Layout {
  static constexpr bool THERMAL = TH;
  static constexpr int LSET = LS;
  static constexpr int V = 14 + (TH ? 3 : 0) + LS;
};

// ---------------------------------------------------------------------------
// Batched form: many independent 1D grids (instances) of uneven sizes, each
// with its own material and its own clock, packed one after another.  For
// instance k with nx_k interior cells the packed index spaces are
//   u  cells   off_u[k]  .. off_u[k]  + nx_k      (off_u[k+1] = off_u[k] + nx_k)
//   ub cells   off_ub[k] .. off_ub[k] + nx_k + 2N (= off_u[k] + 2N k)
//   predictor  off_b[k]  .. off_b[k]  + nx_k + 2  (= off_u[k] + 2 k)
//   faces      off_f[k]  .. off_f[k]  + nx_k + 1  (= off_u[k] + k)
// and inst_* map every packed index to its instance.  clk[k] holds
// {t, dt, tf, cfl, count}; a finished instance has dt = 0 and its steps
// change nothing.
struct Batch {
  const DevPar *P;
  const int32_t *inst_u, *inst_ub, *inst_b, *inst_f;
  const int32_t *nx, *off_u, *off_ub, *off_b, *off_f, *bc;
  const double *idx;  // 1 / dx per instance
  double *clk;        // [ninst][5]
  int ninst;
};

// ---------------------------------------------------------------------------
// Boundary ghost cells (etc/grid.cpp:12-170).  One thread per (ghost row, k)
// of one axis; 2D runs the x pass over interior rows, then the y pass over
// all rows (corners are filled from x ghosts as in the reference).

GPR_D int bc_src_index(int code, int side, int i, int n) {
  // index into the interior line of length n for ghost i (0..N-1) of side
  if (code == GPR_BC_TRANSMISSIVE)
    return side == 0 ? 0 : n - 1;
  if (code == GPR_BC_PERIODIC)
    return side == 0 ? n - NN + i : i;
  return side == 0 ? NN - 1 - i : n - 1 - i;  // reflecting types
}

template <int V>
GPR_D double bc_value(int code, int d, int k, const double *src) {
  double x = src[k];
  switch (code) {
  case GPR_BC_SLIP:
  case GPR_BC_SYMMETRIC:
    if (k == 2 + d)
      x = -x;
    if (code == GPR_BC_SYMMETRIC && k >= 5 && k < 14) {
      int r = (k - 5) / 3, c = (k - 5) % 3;
      if (r == d)
        x = -x;
      if (c == d)
        x = -x;
    }
    break;
  case GPR_BC_STICK:
    if (k >= 2 && k < 5)
      x = -x;
    break;
  case GPR_BC_MOVING:
    if (k >= 2 && k < 5)
      x = -x;
    if (k == 2)
      x += 2.0 * src[0];
    if (k == 1) {
      double m = -src[2] + 2.0 * src[0];
      x += (m * m - src[2] * src[2]) / (2.0 * src[0]);
    }
    break;
  default:
    break;
  }
  return x;
}

// Copies interior u into ub (cell-major), one thread per (cell, var).
template <int V>
__global__ void k_fill_interior(const double *__restrict__ u, double *__restrict__ ub,
                                int nx, int ny, int nd) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  long total = (long)nx * ny * V;
  if (idx >= total)
    return;
  int k = idx % V;
  long c = idx / V;
  if (nd == 1) {
    ub[(c + NN) * V + k] = u[idx];
  } else {
    int i = c / ny, j = c % ny;
    ub[((long)(i + NN) * (ny + 2 * NN) + (j + NN)) * V + k] = u[idx];
  }
}

// 1D boundaries in one launch: ub[p] for p in 0..nx+2N-1, interior cells
// copied from u, ghost cells by the boundary rule from their source cell of u
// (the values k_fill_interior + k_ghosts give), one thread per (cell, var).
template <int V>
__global__ void k_boundaries1d(const double *__restrict__ u, double *__restrict__ ub, int nx,
                               int bcl, int bcr) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)(nx + 2 * NN) * V)
    return;
  const int k = idx % V, p = idx / V;
  if (p >= NN && p < nx + NN) {
    ub[idx] = u[(long)(p - NN) * V + k];
    return;
  }
  const int side = p >= nx + NN;
  const int i = side ? p - nx - NN : p;
  int code = side ? bcr : bcl;
  const int si = bc_src_index(code, side, i, nx);
  if (code == GPR_BC_PERIODIC)
    code = GPR_BC_TRANSMISSIVE;  // plain copy
  ub[idx] = bc_value<V>(code, 0, k, u + (long)si * V);
}

// Ghost rows along one axis.  For axis 0: lines are columns j (interior rows
// j+N of ub when nd == 2), for axis 1: lines are all ub rows i.
template <int V>
__global__ void k_ghosts(double *__restrict__ ub, int nx, int ny, int nd, int axis,
                         int bcl, int bcr) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int nline = nd == 1 ? 1 : (axis == 0 ? ny : nx + 2 * NN);
  long total = (long)nline * 2 * NN * V;
  if (idx >= total)
    return;
  int k = idx % V;
  long rest = idx / V;
  int g = rest % (2 * NN);  // ghost slot: 0..N-1 left, N..2N-1 right
  int line = rest / (2 * NN);
  int side = g >= NN;
  int i = side ? g - NN : g;
  int n = axis == 0 ? nx : ny;
  int code = side ? bcr : bcl;
  int si = bc_src_index(code, side, i, n);
  int gi = side ? i + n + NN : i;  // ghost position along the line
  long nyb = ny + 2 * NN;
  const double *src;
  double *dst;
  if (nd == 1) {
    src = ub + (long)(si + NN) * V;
    dst = ub + (long)gi * V;
  } else if (axis == 0) {
    long j = line + NN;
    src = ub + ((long)(si + NN) * nyb + j) * V;
    dst = ub + ((long)gi * nyb + j) * V;
  } else {
    long ii = line;
    src = ub + (ii * nyb + (si + NN)) * V;
    dst = ub + (ii * nyb + gi) * V;
  }
  if (code == GPR_BC_PERIODIC)
    code = GPR_BC_TRANSMISSIVE;  // plain copy
  dst[k] = bc_value<V>(code, axis, k, src);
}

// ---------------------------------------------------------------------------
// WENO (solvers/weno/weno.cpp:4-124).  One thread per (cell, variable):
// data rows d0[0], d0[sd], d0[2 sd] (cells i-1, i, i+1); writes the N = 2
// node values out[0], out[so].
GPR_D void weno_point(const double *__restrict__ d0, long sd, double *__restrict__ out,
                      long so, int ind, int nx, int gap, const Consts &C) {
  double a = d0[0], b = d0[sd], c = d0[2 * sd];
  double wL0 = C.mLinv[0][0] * a + C.mLinv[0][1] * b;
  double wL1 = C.mLinv[1][0] * a + C.mLinv[1][1] * b;
  double wR0 = C.mRinv[0][0] * b + C.mRinv[0][1] * c;
  double wR1 = C.mRinv[1][0] * b + C.mRinv[1][1] * c;
  // (w^T SIG) w, the reference's evaluation order (weno.cpp:9), which stays
  // accurate on nearly constant data
  double tL = (wL0 * C.sig[0][0] + wL1 * C.sig[1][0]) * wL0 +
              (wL0 * C.sig[0][1] + wL1 * C.sig[1][1]) * wL1 + WENO_EPS;
  double tR = (wR0 * C.sig[0][0] + wR1 * C.sig[1][0]) * wR0 +
              (wR0 * C.sig[0][1] + wR1 * C.sig[1][1]) * wR1 + WENO_EPS;
  tL *= tL;
  tL *= tL;
  tL *= tL;
  tR *= tR;
  tR *= tR;
  tR *= tR;
  const bool useL = ind >= gap, useR = ind <= nx - gap - 1;
  if (useL && useR) {
    // weights LAMS / tL, LAMS / tR normalised, i.e. tR / (tL + tR) and
    // tL / (tL + tR): one division where the reference takes three (equal
    // side weights; the result moves by an ulp at most)
    static_assert(LAMS == 1.0, "equal side weights");
    const double iden = 1.0 / (tL + tR);
    out[0] = (wL0 * tR + wR0 * tL) * iden;
    out[so] = (wL1 * tR + wR1 * tL) * iden;
    return;
  }
  double oL = LAMS / tL, oR = LAMS / tR;
  double n0 = 0.0, n1 = 0.0, den = 0.0;
  if (useL) {
    n0 += wL0 * oL;
    n1 += wL1 * oL;
    den += oL;
  }
  if (useR) {
    n0 += wR0 * oR;
    n1 += wR1 * oR;
    den += oR;
  }
  double iden = 1.0 / den;
  out[0] = n0 * iden;
  out[so] = n1 * iden;
}

// 1D: wh[i][a][k] for i in 0..nx+1 from ub rows i..i+2 (weno.cpp:75-81, 146)
template <int V>
__global__ void k_weno1d(double *__restrict__ wh, const double *__restrict__ ub, int ncb,
                         Consts C) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)ncb * V)
    return;
  int k = idx % V;
  int i = idx / V;
  weno_point(ub + (long)i * V + k, V, wh + (long)i * NN * V + k, V, i, ncb, 0, C);
}

// 2D, both sweeps in one launch, staged in shared memory: a block takes
// predictor row i (one of nx+2) and output columns j0 .. j0+jn-1 (jn <= tj).
// It loads the jn+2 ub columns of ub rows i, i+1, i+2 that the x sweep
// reads (each row segment is contiguous in the cell-major layout: 16-byte
// loads, with single doubles only at an unaligned start or end), runs the x
// sweep on them into a shared ux tile (node a = 0, 1 of each column), and
// the y sweep of its jn columns from that tile into wh.  Each point is
// weno_point with the reference's one-sided edges (weno.cpp:93-121); the
// x sweep's 2 edge columns of a tile are evaluated again by its neighbour
// tile.  ux never reaches global memory.
constexpr int WENO2_COLS = 64, WENO2_THREADS = 256;
template <int V>
__global__ void __launch_bounds__(WENO2_THREADS) k_weno2d(double *__restrict__ wh,
                                                         const double *__restrict__ ub,
                                                         int nxp, int nyp, int tj, Consts C) {
  constexpr int RS = WENO2_COLS * V;  // shared row stride (doubles)
  __shared__ double sub[3 * RS];
  __shared__ double sux[WENO2_COLS * NN * V];
  const int nyb = nyp + 2 * (NN - 1);
  const int nbj = (nyp + tj - 1) / tj;
  const int i = blockIdx.x / nbj, j0 = (blockIdx.x % nbj) * tj;
  const int jn = min(tj, nyp - j0), nc = jn + 2;
  const int len = nc * V;
  // 1. stage ub rows i .. i+2, columns j0 .. j0+nc-1
  for (int r = 0; r < 3; r++) {
    const double *src = ub + ((long)(i + r) * nyb + j0) * V;
    const int off = (int)(((unsigned long long)src >> 3) & 1);  // src not 16-byte aligned
    const int npair = (off + len + 1) / 2;
    double *dst = sub + r * RS;
    for (int p = threadIdx.x; p < npair; p += WENO2_THREADS) {
      const int lo = 2 * p - off;  // element index of the pair's first double
      if (lo >= 0 && lo + 1 < len) {
        const double2 x = *reinterpret_cast<const double2 *>(src + lo);
        dst[lo] = x.x;
        dst[lo + 1] = x.y;
      } else {
        if (lo >= 0)
          dst[lo] = src[lo];
        if (lo + 1 >= 0 && lo + 1 < len)
          dst[lo + 1] = src[lo + 1];
      }
    }
  }
  __syncthreads();
  // 2. x sweep (weno.cpp:93-104) of the nc staged columns
  for (int e = threadIdx.x; e < len; e += WENO2_THREADS) {
    const int c = e / V, k = e % V;
    const int j = j0 + c;
    const int gap = (j < NN || j >= nyb - NN) ? NN : 0;
    weno_point(sub + c * V + k, RS, sux + c * NN * V + k, V, i, nxp, gap, C);
  }
  __syncthreads();
  // 3. y sweep (weno.cpp:106-121) of the jn output columns
  const int gap = (i == 0 || i == nxp - 1) ? 1 : 0;
  for (int e = threadIdx.x; e < jn * NN * V; e += WENO2_THREADS) {
    const int k = e % V, a = (e / V) % NN, c = e / (NN * V);
    const int j = j0 + c;
    weno_point(sux + (c * NN + a) * V + k, (long)NN * V,
               wh + (((long)i * nyp + j) * NN * NN + a * NN) * V + k, V, j, nyp, gap, C);
  }
}

// Output columns per k_weno2d block: at most WENO2_COLS - 2, spread evenly
// over the row's blocks.
inline int weno2d_tile(int nyp) {
  const int nbj = (nyp + WENO2_COLS - 3) / (WENO2_COLS - 2);
  return (nyp + nbj - 1) / nbj;
}

// Sum an n-vector v over the G lanes of each aligned lane group (xor
// butterfly) and scatter the sum: afterwards lane r = lane % G holds
// elements r n/G .. (r + 1) n/G - 1 of the sum in v[0 .. n/G - 1].  At each
// level a lane keeps one half, chosen by its lane bit (a select: integer
// work), and adds the partner's copy of it, so a lane issues n/2 + n/4 + ...
// + n/G FP64 adds where a full butterfly issues n log2 G; on this GPU the
// FP64 cost is per warp instruction, whatever the active lanes.
template <int n, int G> struct GroupReduceScatter {
  static_assert(n % G == 0, "n a multiple of G");
  static GPR_D void run(double *v, int r) {
    if constexpr (G > 1) {
      constexpr int h = n / 2;
      const bool up = r & (G / 2);
#pragma unroll
      for (int j = 0; j < h; j++) {
        const double keep = up ? v[h + j] : v[j];
        const double send = up ? v[j] : v[h + j];
        v[j] = keep + __shfl_xor_sync(0xffffffffu, send, G / 2);
      }
      GroupReduceScatter<h, G / 2>::run(v, r);
    }
  }
};

// The face contributions kk (b + f) (left cell) and kk (b - f) (right cell)
// summed over the G quadrature lanes of a face (r = lane within the face)
// and written to out[0..V-1] / out[V..2V-1] by the lanes that hold them.
template <int V, int G>
GPR_D void face_reduce_store(const double *b, const double *f, double kk, bool active,
                             bool valid, int r, double *out) {
  constexpr int NPR = (V + G - 1) / G;  // (b, f) pairs per lane after the scatter
  double v[2 * NPR * G];
#pragma unroll
  for (int k = 0; k < NPR * G; k++) {
    v[2 * k] = (active && k < V) ? kk * b[k] : 0.0;
    v[2 * k + 1] = (active && k < V) ? kk * f[k] : 0.0;
  }
  GroupReduceScatter<2 * NPR * G, G>::run(v, r);
  if (!valid)
    return;
#pragma unroll
  for (int p = 0; p < NPR; p++) {
    const int k = r * NPR + p;
    if (k < V) {
      out[k] = v[2 * p] + v[2 * p + 1];
      out[V + k] = v[2 * p] - v[2 * p + 1];
    }
  }
}

// The same sums applied to the state in place (interfs1 / interfs2 update u
// inside the face loop, fv.cpp:143-146, 217-222, 257-262): uL -= out[0..V-1]
// on the cell to the left of the face, uR -= out[V..2V-1] on the cell to its
// right (either may be null: no interior cell there).  Only for faces with
// face_on (the face's own activity: geometry and mask, not the lane's).
template <int V, int G>
GPR_D void face_reduce_apply(const double *b, const double *f, double kk, bool active,
                             bool face_on, int r, double *uL, double *uR) {
  constexpr int NPR = (V + G - 1) / G;
  double v[2 * NPR * G];
#pragma unroll
  for (int k = 0; k < NPR * G; k++) {
    v[2 * k] = (active && k < V) ? kk * b[k] : 0.0;
    v[2 * k + 1] = (active && k < V) ? kk * f[k] : 0.0;
  }
  GroupReduceScatter<2 * NPR * G, G>::run(v, r);
  if (!face_on)
    return;
#pragma unroll
  for (int p = 0; p < NPR; p++) {
    const int k = r * NPR + p;
    if (k < V) {
      if (uL)
        uL[k] -= v[2 * p] + v[2 * p + 1];
      if (uR)
        uR[k] -= v[2 * p] - v[2 * p + 1];
    }
  }
}

// Faces of one 2D face pass.  parity < 0: every face (i, j) of the
// (nx+1) x (ny+1) face grid of direction dir.  parity 0 / 1: only the faces
// whose index along dir has that parity; two such faces never share a cell,
// so a pass can update u in place without races, and the four passes
// (direction x parity) cover every face once.
struct Face2 {
  long fi;    // flat face index (i (ny + 1) + j)
  int i, j;   // predictor-cell indices of the face's left / lower cell
  bool valid;
};
GPR_HD long face2_count(int nx, int ny, int dir, int parity) {
  if (parity < 0)
    return (long)(nx + 1) * (ny + 1);
  return dir == 0 ? (long)((nx + 2 - parity) / 2) * (ny + 1)
                  : (long)(nx + 1) * ((ny + 2 - parity) / 2);
}
GPR_D Face2 face2_of(long face, int nx, int ny, int dir, int parity) {
  Face2 F;
  F.valid = face < face2_count(nx, ny, dir, parity);
  long e = F.valid ? face : 0;
  if (parity < 0) {
    F.i = e / (ny + 1);
    F.j = e % (ny + 1);
  } else if (dir == 0) {
    F.i = 2 * (int)(e / (ny + 1)) + parity;
    F.j = e % (ny + 1);
  } else {
    const int nfj = (ny + 2 - parity) / 2;
    F.i = e / nfj;
    F.j = 2 * (int)(e % nfj) + parity;
  }
  F.fi = (long)F.i * (ny + 1) + F.j;
  return F;
}
// The interior cells on either side of face (i, j) of direction dir, as
// pointers into u[nx][ny][V] (null where the side is a ghost cell).
GPR_D void face2_cells(double *u, int i, int j, int nx, int ny, int dir, int V, double *&uL,
                       double *&uR) {
  if (dir == 0) {
    uL = i >= 1 ? u + ((long)(i - 1) * ny + (j - 1)) * V : nullptr;
    uR = i <= nx - 1 ? u + ((long)i * ny + (j - 1)) * V : nullptr;
  } else {
    uL = j >= 1 ? u + ((long)(i - 1) * ny + (j - 1)) * V : nullptr;
    uR = j <= ny - 1 ? u + ((long)(i - 1) * ny + j) * V : nullptr;
  }
}

// ---------------------------------------------------------------------------
// Space-time DG predictor (solvers/dg/dg1.cpp:8-114, dg2.cpp:8-171).
//
// One thread per space-time node: NP = N^(d+1) consecutive lanes hold one
// cell (lane g = t N^d + s).  Spatial derivatives, the DG_DER flux term and
// the DG_U^-1 time coupling need the partner nodes' values, exchanged with
// warp shuffles (partners differ in one index: lane ^ bit).  Each iteration
// is the reference's Picard update q <- DG_U^-1 (Ww + dt R(q)) with its
// per-cell stopping rule |q1 - q0| <= dg_tol (1 + |q0|) (dg1.cpp:91-110).

// |x| as the bit pattern of a non-negative double; patterns above
// FP_INF_BITS are NaNs.
constexpr unsigned long long FP_INF_BITS = 0x7ff0000000000000ULL;
// growth of a cell's largest Picard update over its smallest that hands the
// cell to the Newton pass (k_predictor_picard)
constexpr double PICARD_DIVERGE = 1e3;
GPR_D unsigned long long fp_abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}

template <int V>
GPR_D void shfl_vec(const double *src, double *dst, int lanemask) {
#pragma unroll
  for (int k = 0; k < V; k++)
    dst[k] = __shfl_xor_sync(0xffffffffu, src[k], lanemask);
}

// rhs at this thread's node with time weight wt (W_t): r = dt R + Ww
// (AFFINE) or r = R; q unchanged.  The spatial partners are the lanes
// g ^ XB (x) and g ^ YB (y), as in both lane layouts that call it.
template <class L, int ND, bool AFFINE = true>
GPR_D void dg_rhs_node_w(const double *q, const double *Ww, double *r, double wt, int i, int j,
                         double dt, double idx, double idy, const DevPar &P, const Consts &C) {
  constexpr int V = L::V;
  // lane bit layout: 1D g = 2t + i ; 2D g = 4t + 2i + j
  constexpr int XB = ND == 1 ? 1 : 2;  // flips i
  constexpr int YB = 1;                // flips j (2D)
  double tmp[V], other[V];
  Prim<L::THERMAL> s;
  prim<L::THERMAL>(q, P, s);
  // W (S - B dq/dx [- B dq/dy]): the node weight wn folded into the
  // source's scalar factors and the derivative coefficients (B is linear)
  const double wn = ND == 1 ? wt * C.w[i] : wt * C.w[i] * C.w[j];
  source<L::THERMAL, V>(q, s, P, r, wn);
  // x derivative: DERVALS[i][m] q(t, m, j) / dx
  shfl_vec<V>(q, other, XB);
  {
    double a = C.derv[i][i] * idx * wn, b = C.derv[i][1 - i] * idx * wn;
#pragma unroll
    for (int k = 0; k < V; k++)
      tmp[k] = a * q[k] + b * other[k];
    double bd[V];
    bdot<V, L::LSET>(s.v, tmp, 0, bd);
#pragma unroll
    for (int k = 0; k < V; k++)
      r[k] -= bd[k];
  }
  if (ND == 2) {
    shfl_vec<V>(q, other, YB);
    double a = C.derv[j][j] * idy * wn, b = C.derv[j][1 - j] * idy * wn;
#pragma unroll
    for (int k = 0; k < V; k++)
      tmp[k] = a * q[k] + b * other[k];
    double bd[V];
    bdot<V, L::LSET>(s.v, tmp, 1, bd);
#pragma unroll
    for (int k = 0; k < V; k++)
      r[k] -= bd[k];
  }
  // - W_t [W_j] DG_DER(i, m) F(t, m, j) / dx, as two fused multiply-adds
  flux_set<L::THERMAL, V>(q, s, 0, P, tmp);
  shfl_vec<V>(tmp, other, XB);
  {
    double wx = (ND == 1 ? wt : wt * C.w[j]) * idx;
    double a = wx * C.dgder[i][i], b = wx * C.dgder[i][1 - i];
#pragma unroll
    for (int k = 0; k < V; k++)
      if (flux_support<L::THERMAL>(k, 0))
        r[k] = fma(-b, other[k], fma(-a, tmp[k], r[k]));
  }
  if (ND == 2) {
    flux_set<L::THERMAL, V>(q, s, 1, P, tmp);
    shfl_vec<V>(tmp, other, YB);
    double wy = wt * C.w[i] * idy;
    double a = wy * C.dgder[j][j], b = wy * C.dgder[j][1 - j];
#pragma unroll
    for (int k = 0; k < V; k++)
      if (flux_support<L::THERMAL>(k, 1))
        r[k] = fma(-b, other[k], fma(-a, tmp[k], r[k]));
  }
  if (AFFINE) {
#pragma unroll
    for (int k = 0; k < V; k++)
      r[k] = r[k] * dt + Ww[k];
  }
}

template <class L, int ND>
GPR_D void dg_rhs_node(const double *q, const double *Ww, double *r, int t, int i, int j,
                       double dt, double idx, double idy, const DevPar &P, const Consts &C) {
  dg_rhs_node_w<L, ND, true>(q, Ww, r, C.w[t], i, j, dt, idx, idy, P, C);
}

// q_new(t, s) = sum_m DG_MATinv[t][m] r(m, s) / W_s
template <int V, int ND>
GPR_D void dg_solve_node(const double *r, double *qn, int t, int i, int j, const Consts &C) {
  constexpr int TB = ND == 1 ? 2 : 4;  // flips t
  double other[V];
  shfl_vec<V>(r, other, TB);
  // 1 / W_s: 2 and 4 for the N = 2 weights (exact)
  double iws = ND == 1 ? 1.0 / C.w[i] : 1.0 / (C.w[i] * C.w[j]);
  double a = C.dgmatinv[t][t] * iws, b = C.dgmatinv[t][1 - t] * iws;
#pragma unroll
  for (int k = 0; k < V; k++)
    qn[k] = a * r[k] + b * other[k];
}

// First Picard iteration.  From the standard initial guess q(t, s) = w(s)
// (initial_guess.cpp:4-15) the rhs at the two time nodes differs only by the
// weight W_t, so one thread per (cell, spatial node) evaluates it once (time
// weight 1) and writes q1 = DG_U^-1 (W w + dt R(q0)) at both time nodes
// into qh; k_predictor_picard (first = 1) takes that as its first iterate
// and applies the reference's stopping test to it as usual.
template <class L, int ND, bool BATCH = false>
__global__ void __launch_bounds__(128) k_predictor_first(
    double *__restrict__ qh, const double *__restrict__ wh, long ncb,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double idx,
    double idy, DevPar Pv, Consts C, Batch B) {
  constexpr int V = L::V;
  constexpr int NS = ND == 1 ? NN : NN * NN;  // spatial nodes
  constexpr int NP = NN * NS;
  static_assert(NN == 2, "two time nodes");
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int g = threadIdx.x % NS;
  long c = gt / NS;
  bool valid = c < ncb;
  const long cc = valid ? c : 0;
  const int inst = BATCH ? B.inst_b[cc] : 0;
  const DevPar &P = BATCH ? B.P[inst] : Pv;
  if (BATCH) {
    dt = B.clk[5 * inst + 1];
    idx = B.idx[inst];
  }
  // the cells k_predictor_picard iterates (finished instances of a batch too)
  const bool active = valid && (mask == nullptr || mask[c]);
  const int i = ND == 1 ? g : g / NN, j = ND == 1 ? 0 : g % NN;
  double q[V], r[V];
  const double *wc = wh + (cc * NS + g) * V;
#pragma unroll
  for (int k = 0; k < V; k++)
    q[k] = valid ? wc[k] : 1.0;
  dg_rhs_node_w<L, ND, false>(q, nullptr, r, 1.0, i, j, dt, idx, idy, P, C);
  if (!active)
    return;
  // r_t = dt W_t R + ENDVALS[0][t] W_s w ; q1_t = sum_m DG_MATinv[t][m] r_m / W_s
  const double Ws = ND == 1 ? C.w[i] : C.w[i] * C.w[j];
  const double iws = ND == 1 ? 1.0 / C.w[i] : 1.0 / (C.w[i] * C.w[j]);
  const double d0 = dt * C.w[0], d1 = dt * C.w[1];
  const double f0 = C.endv[0][0] * Ws, f1 = C.endv[0][1] * Ws;
  const double a00 = C.dgmatinv[0][0] * iws, a01 = C.dgmatinv[0][1] * iws;
  const double a10 = C.dgmatinv[1][0] * iws, a11 = C.dgmatinv[1][1] * iws;
  double *o0 = qh + (c * NP + g) * V, *o1 = qh + (c * NP + NS + g) * V;
#pragma unroll
  for (int k = 0; k < V; k++) {
    const double r0 = r[k] * d0 + f0 * q[k];
    const double r1 = r[k] * d1 + f1 * q[k];
    o0[k] = a00 * r0 + a01 * r1;
    o1[k] = a10 * r0 + a11 * r1;
  }
}

// Picard predictor.  ncb predictor cells; each warp holds 32/NP cells.
// status[c] (optional): GPR_PRED_PICARD | iterations << 8 when converged,
// GPR_PRED_FAILED when Picard did not converge (row left for the Newton pass,
// with the last Picard iterate written so the row is always defined).
struct PicardResume {
  int cap = 0;
  int *list = nullptr, *n = nullptr;
  int *it = nullptr;
  double *dmin = nullptr;
  const int *in = nullptr, *n_in = nullptr;
};

template <class L, int ND, bool BATCH = false>
__global__ void __launch_bounds__(128) k_predictor_picard(
    double *__restrict__ qh, const double *__restrict__ wh, long ncb,
    const uint8_t *__restrict__ mask, int32_t *__restrict__ status, double dt,
    const double *__restrict__ dt_dev, double idx, double idy, int stiff, DevPar Pv, Consts C,
    Batch B, int first, PicardResume R = PicardResume{}) {
  constexpr int V = L::V;
  constexpr int NS = ND == 1 ? NN : NN * NN;  // spatial nodes
  constexpr int NP = NN * NS;                 // space-time nodes
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int g = threadIdx.x % NP;
  long c = gt / NP;
  bool valid = c < ncb;
  if (R.in) {
    const long qi = gt / NP;
    valid = qi < *R.n_in;
    c = valid ? R.in[qi] : 0;
  }
  const int inst = BATCH ? B.inst_b[valid ? c : 0] : 0;
  const DevPar &P = BATCH ? B.P[inst] : Pv;
  if (BATCH) {
    dt = B.clk[5 * inst + 1];
    idx = B.idx[inst];
  }
  bool active = valid && (mask == nullptr || mask[c]);
  int t = g / NS, sidx = g % NS;
  int i = ND == 1 ? sidx : sidx / NN, j = ND == 1 ? 0 : sidx % NN;
  double w[V], Ww[V], q[V], r[V], qn[V];
  long cc = valid ? c : 0;
  const double *wc = wh + (cc * NS + sidx) * V;
  double f = C.endv[0][t] * (ND == 1 ? C.w[i] : C.w[i] * C.w[j]);
#pragma unroll
  for (int k = 0; k < V; k++) {
    w[k] = valid ? wc[k] : 1.0;
    Ww[k] = f * w[k];
    q[k] = (R.in && valid) ? qh[(cc * NP + g) * V + k] : w[k];
  }
  // groups are aligned to NP lanes; the group shares the convergence decision
  unsigned lane = threadIdx.x & 31u;
  unsigned gmask = ((NP == 32) ? 0xffffffffu : ((1u << NP) - 1u)) << (lane & ~(NP - 1u));
  bool done = !active;
  int iters = 0;
  bool nan_seen = false;
  const int maxit = stiff ? 0 : C.dg_it;
  // Divergence detection: a cell whose largest update has grown DIVERGE
  // times above the smallest it reached is diverging and goes to the
  // stiff-source Newton pass at once instead of spending the rest of the
  // iteration cap.  Measured with the oracle's Picard iteration over
  // 2D TGV states at CFL 0.4 .. 1.0, stiff 1D tubes and the batched
  // instances: cells that converge (some only after ~40 iterations) grow by
  // at most 4.3x before converging, cells that fail grow past 1e3 within
  // 4 .. 25 iterations and saturate near O(1) updates (without this test
  // they run the whole cap of 50).  So every cell the reference's Picard
  // iteration converges still converges by Picard.
  const bool resume = R.in != nullptr && valid;
  const int it0 = resume ? R.it[c] : 0;
  double dmin = resume ? R.dmin[c] : 1e300;
  bool failed = false, deferred = false;
  for (int kq = 0;; kq++) {
    const int it = it0 + kq;
    if (!done && it >= maxit) {
      failed = true;
      done = true;
    }
    if (!done && R.cap > 0 && kq == R.cap) {
      double *outd = qh + (c * NP + g) * V;
#pragma unroll
      for (int k = 0; k < V; k++)
        outd[k] = q[k];
      if (g == 0) {
        R.it[c] = it;
        R.dmin[c] = dmin;
        R.list[atomicAdd(R.n, 1)] = (int)c;
      }
      deferred = true;
      done = true;
    }
    if (__all_sync(0xffffffffu, done))
      break;
    // (a continuation never takes this branch, not even on its unused lanes,
    // whose it0 is 0: the other branch's shuffles need the whole warp)
    if (it == 0 && first && R.in == nullptr) {
      // the first iterate, from k_predictor_first
      const double *src = qh + (cc * NP + g) * V;
#pragma unroll
      for (int k = 0; k < V; k++)
        qn[k] = active ? src[k] : q[k];
    } else {
      dg_rhs_node<L, ND>(q, Ww, r, t, i, j, dt, idx, idy, P, C);
      dg_solve_node<V, ND>(r, qn, t, i, j, C);
    }
    // the reference's test |q1 - q0| > dg_tol (1 + |q0|) per entry, the
    // comparisons and maxima on the IEEE bit patterns of the non-negative
    // operands (integer order equals numeric order there; NaN patterns sort
    // above infinity and are excluded as the floating-point forms exclude
    // them), so that only the subtraction and the threshold use the FP64 pipe
    bool big = false, hasnan = false;
    unsigned long long dmaxb = 0;
#pragma unroll
    for (int k = 0; k < V; k++) {
      const unsigned long long ddb = fp_abs_bits(qn[k] - q[k]);
      const unsigned long long thb = fp_abs_bits(C.dg_tol * (1.0 + fabs(q[k])));
      if (ddb > thb && ddb <= FP_INF_BITS && thb <= FP_INF_BITS)
        big = true;
      if (fp_abs_bits(qn[k]) > FP_INF_BITS)
        hasnan = true;
      if (ddb <= FP_INF_BITS && ddb > dmaxb)
        dmaxb = ddb;
    }
#pragma unroll
    for (int o = 1; o < NP; o <<= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, dmaxb, o);
      dmaxb = x > dmaxb ? x : dmaxb;
    }
    const double dmax = __longlong_as_double((long long)dmaxb);
    unsigned bigm = __ballot_sync(0xffffffffu, big) & gmask;
    unsigned nanm = __ballot_sync(0xffffffffu, hasnan) & gmask;
    if (!done && bigm && it >= 3 && dmax > PICARD_DIVERGE * dmin) {
      nan_seen = true;  // hand over to the Newton pass
      done = true;
      iters = it + 1;
    }
    if (!done)
      dmin = dmax < dmin ? dmax : dmin;
    if (!done) {
      iters = it + 1;
      if (bigm) {
#pragma unroll
        for (int k = 0; k < V; k++)
          q[k] = qn[k];
      } else if (nanm) {
        nan_seen = true;
        done = true;
      } else {
#pragma unroll
        for (int k = 0; k < V; k++)
          q[k] = qn[k];
        done = true;
        if (active) {
          double *out = qh + (c * NP + g) * V;
#pragma unroll
          for (int k = 0; k < V; k++)
            out[k] = q[k];
          if (status && g == 0)
            status[c] = GPR_PRED_PICARD | (iters << 8);
        }
      }
    }
  }
  if (active && !deferred && (failed || nan_seen)) {
    // Picard failed: write the initial guess and flag the cell for the
    // stiff-source Newton pass with a NaN in its first entry
    double *out = qh + (c * NP + g) * V;
#pragma unroll
    for (int k = 0; k < V; k++)
      out[k] = w[k];
    if (g == 0)
      out[0] = __longlong_as_double(0x7ff8000000000bad);
    if (status && g == 0)
      status[c] = GPR_PRED_FAILED | (iters << 8);
  }
  if (valid && !active && status && g == 0)
    status[c] = GPR_PRED_PICARD;
}

// ---------------------------------------------------------------------------
// midstepper (split/homogeneous.cpp:5-67): the half step of the homogeneous
// system at the WENO nodes before the split scheme's FV update,
//   w_s -= dt/2 ((dF/dx + B_x dw/dx) / dx [+ (dG/dy + B_y dw/dy) / dy]),
// derivatives by DERVALS within the cell.  One thread per spatial node, the
// cell's NS = N^d lanes adjacent (x partner lane ^ (ND == 1 ? 1 : 2), y
// partner lane ^ 1).
template <class L, int ND>
__global__ void __launch_bounds__(128) k_midstep(double *__restrict__ wh, long ncb,
                                                 const uint8_t *__restrict__ mask, double dt,
                                                 const double *__restrict__ dt_dev, double idx,
                                                 double idy, DevPar P, Consts C) {
  constexpr int V = L::V;
  constexpr int NS = ND == 1 ? NN : NN * NN;
  constexpr int XB = ND == 1 ? 1 : 2, YB = 1;
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int g = threadIdx.x % NS;
  const long c = gt / NS;
  const bool valid = c < ncb;
  const long cc = valid ? c : 0;
  const bool active = valid && (mask == nullptr || mask[cc]);
  const int a = ND == 1 ? g : g / NN, b = ND == 1 ? 0 : g % NN;
  double w[V], F[V], other[V], dw[V], inc[V];
  double *wc = wh + (cc * NS + g) * V;
#pragma unroll
  for (int k = 0; k < V; k++)
    w[k] = wc[k];
  Prim<L::THERMAL> s;
  prim<L::THERMAL>(w, P, s);
#pragma unroll
  for (int k = 0; k < V; k++)
    F[k] = 0.0;
  flux_add<L::THERMAL, V>(w, s, 0, P, F);
  // x: d/dx of w and F over the x partner
  {
    const double ca = C.derv[a][a], cb = C.derv[a][1 - a];
    shfl_vec<V>(w, other, XB);
#pragma unroll
    for (int k = 0; k < V; k++)
      dw[k] = ca * w[k] + cb * other[k];
    shfl_vec<V>(F, other, XB);
    double bd[V];
    bdot<V, L::LSET>(s.v, dw, 0, bd);
#pragma unroll
    for (int k = 0; k < V; k++)
      inc[k] = ((ca * F[k] + cb * other[k]) + bd[k]) * idx;
  }
  if (ND == 2) {
    const double ca = C.derv[b][b], cb = C.derv[b][1 - b];
#pragma unroll
    for (int k = 0; k < V; k++)
      F[k] = 0.0;
    flux_add<L::THERMAL, V>(w, s, 1, P, F);
    shfl_vec<V>(w, other, YB);
#pragma unroll
    for (int k = 0; k < V; k++)
      dw[k] = ca * w[k] + cb * other[k];
    shfl_vec<V>(F, other, YB);
    double bd[V];
    bdot<V, L::LSET>(s.v, dw, 1, bd);
#pragma unroll
    for (int k = 0; k < V; k++)
      inc[k] += ((ca * F[k] + cb * other[k]) + bd[k]) * idy;
  }
  if (active) {
#pragma unroll
    for (int k = 0; k < V; k++)
      wc[k] = w[k] - dt / 2 * inc[k];
  }
}

// ---------------------------------------------------------------------------
// Stiff-source Newton pass for the cells whose Picard iteration failed (the
// reference leaves their rows unwritten, dg1.cpp:91-110, or falls back to a
// Jacobian-free Newton-Krylov solve on NaN, dg1.cpp:100-105).
//
// Iteration on the predictor fixed point Fp(q) = DG_U q - Ww - dt R(q) = 0:
//   delta = (DG_U - dt W dS/dq)^-1 (Ww + dt R(q) - DG_U q),   q += delta,
// with dS/dq the exact local Jacobian of the relaxation sources at each
// space-time node (distortion 9x9, heat flux 3x3): implicit in the stiff
// sources, explicit in the fluxes; with dS/dq = 0 it is the Picard update.
// Per spatial node the correction couples the N = 2 time nodes through
// DG_MAT: an 18x18 system for A and a 6x6 system for rho J, assembled in
// shared memory by the node's two lanes and solved by one lane each
// (partial pivoting); the other variables use DG_MAT^-1 directly.

template <bool TH>
GPR_D void stiff_jacobian_rows(const double *q, const Prim<TH> &s, const DevPar &P, double a,
                               double mdiag, float *rowsA, int ldA, float *rowsJ, int ldJ) {
  // rowsA[i*ldA + j] (i = 0..8, j = 0..8): M[t][t] delta_ij - a JA[i][j]
  const double *A = q + 5;
  double H[9], dG[9];
  double G00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  double G11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  double G22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  double G01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  double G02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  double G12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  double t3 = (G00 + G11 + G22) * (1.0 / 3.0);
  dG[0] = G00 - t3; dG[1] = G01; dG[2] = G02;
  dG[3] = G01; dG[4] = G11 - t3; dG[5] = G12;
  dG[6] = G02; dG[7] = G12; dG[8] = G22 - t3;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int m = 0; m < 3; m++)
      H[3 * i + m] = A[3 * i] * A[3 * m] + A[3 * i + 1] * A[3 * m + 1] + A[3 * i + 2] * A[3 * m + 2];
  double dA = det3(A);
  int newtonian = !(P.flags & (GPR_SOLID | GPR_POWER_LAW | GPR_BINGHAM));
  double th = theta1inv<TH>(q, s, P);
  double id = 1.0 / dA;
  double Ai[9];  // A^-1
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) * id;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = (A[5] * A[6] - A[3] * A[8]) * id;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) * id;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  double fth = newtonian ? (5.0 / 3.0) * th : 0.0;
  double ca = a * s.cs2;  // a (-JA) = ca (th v + AdG dth)
  // The 81 entries in FP32: the rows are stored in FP32 for the FP32
  // correction solve (the residual stays FP64, so the converged point is the
  // FP64 fixed point), and FP32 runs beside the FP64 pipe at full rate.
  float Af[9], dGf[9], Hf[9], Aif[9], AdGf[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    Af[k] = (float)A[k];
    dGf[k] = (float)dG[k];
    Hf[k] = (float)H[k];
    Aif[k] = (float)(Ai[k] * fth);
    AdGf[k] = (float)(s.AdG[k] * ca);
  }
  const float cth = (float)(ca * th), md = (float)mdiag;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      int rr = 3 * i + j;
#pragma unroll
      for (int m = 0; m < 3; m++)
#pragma unroll
        for (int n = 0; n < 3; n++) {
          float v = (i == m ? dGf[3 * n + j] : 0.0f) + Af[3 * i + n] * Af[3 * m + j] +
                    (n == j ? Hf[3 * i + m] : 0.0f) -
                    (2.0f / 3.0f) * Af[3 * i + j] * Af[3 * m + n];
          float e = cth * v + AdGf[rr] * Aif[3 * n + m];
          rowsA[rr * ldA + 3 * m + n] = (rr == 3 * m + n ? md : 0.0f) + e;
        }
    }
  if (TH) {
    double f = a * P.calpha2 * P.ikappa;  // -a JJ = f (T/rho I + J dT)
#pragma unroll
    for (int l = 0; l < 3; l++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        double dT = -P.calpha2 * s.J[k] * s.ir * P.icv;
        rowsJ[l * ldJ + k] =
            (float)((l == k ? mdiag : 0.0) + f * ((l == k ? s.T * s.ir : 0.0) + s.J[l] * dT));
      }
  }
}

// In-place Gaussian elimination with partial pivoting on the n x n system
// M (leading dimension ld) with right-hand side b; solution left in b.  The
// stiff pass solves its correction systems in FP32: the residual is FP64, so
// the converged fixed point is the FP64 one and the single-precision
// Jacobian only changes the (already linear) contraction rate slightly.
template <int n, class R>
GPR_D bool smem_solve(R *M, int ld, R *b) {
  for (int c = 0; c < n; c++) {
    int p = c;
    R best = fabs(M[c * ld + c]);
#pragma unroll 4
    for (int r = c + 1; r < n; r++) {
      R v = fabs(M[r * ld + c]);
      if (v > best) {
        best = v;
        p = r;
      }
    }
    if (!(best > R(0)))
      return false;
    if (p != c) {
#pragma unroll 4
      for (int j = c; j < n; j++) {
        R tmp = M[c * ld + j];
        M[c * ld + j] = M[p * ld + j];
        M[p * ld + j] = tmp;
      }
      R tmp = b[c];
      b[c] = b[p];
      b[p] = tmp;
    }
    R inv = R(1) / M[c * ld + c];
    for (int r = c + 1; r < n; r++) {
      R f = M[r * ld + c] * inv;
#pragma unroll 4
      for (int j = c + 1; j < n; j++)
        M[r * ld + j] -= f * M[c * ld + j];
      b[r] -= f * b[c];
    }
  }
  for (int r = n - 1; r >= 0; r--) {
    R acc = b[r];
#pragma unroll 4
    for (int j = r + 1; j < n; j++)
      acc -= M[r * ld + j] * b[j];
    b[r] = acc / M[r * ld + r];
  }
  return true;
}

template <class L, int ND> struct StiffSmem {
  static constexpr int NS = ND == 1 ? NN : NN * NN;
  static constexpr int NA = 9 * NN, NJ = 3 * NN;
  // odd number of floats: the solver lanes of neighbouring spatial nodes
  // then start on different shared-memory banks
  static constexpr int raw = NA * NA + NA + (L::THERMAL ? NJ * NJ + NJ : 0);
  static constexpr int per_node = raw | 1;
  static constexpr int CPB = 8;  // cells per 64-thread block (2D: 8 lanes each)
  static constexpr int per_cell = NS * per_node;
};

template <class L, int ND, bool BATCH = false>
__global__ void __launch_bounds__(64) k_predictor_stiff(
    double *__restrict__ qh, const double *__restrict__ wh, long ncb,
    const uint8_t *__restrict__ mask, int32_t *__restrict__ status, double dt_in,
    const double *__restrict__ dt_dev, double idx_in, double idy, DevPar Pv, Consts C,
    Batch B) {
  constexpr int V = L::V;
  constexpr int NS = ND == 1 ? NN : NN * NN;
  constexpr int NP = NN * NS;
  constexpr int TB = ND == 1 ? 2 : 4;  // flips t
  constexpr int NA = 9 * NN, NJ = 3 * NN;
  using SM = StiffSmem<L, ND>;
  extern __shared__ float fsmem[];
  if (dt_dev)
    dt_in = *dt_dev;
  const int g = threadIdx.x % NP;
  const int t = g / NS, sidx = g % NS;
  const int i = ND == 1 ? sidx : sidx / NN, j = ND == 1 ? 0 : sidx % NN;
  float *cellmem = fsmem + (threadIdx.x / NP) * SM::per_cell;
  float *Am = cellmem + sidx * SM::per_node;  // 18 x 18
  float *Ab = Am + NA * NA;                   // 18
  float *Jm = Ab + NA;                        // 6 x 6
  float *Jb = Jm + NJ * NJ;                   // 6
  const unsigned lane = threadIdx.x & 31u;
  const unsigned gmask = ((NP == 32) ? 0xffffffffu : ((1u << NP) - 1u)) << (lane & ~(NP - 1u));
  const double f = C.endv[0][t] * (ND == 1 ? C.w[i] : C.w[i] * C.w[j]);
  const double ws = ND == 1 ? C.w[i] : C.w[i] * C.w[j];
  const double iws = 1.0 / ws;
  const double M0 = C.dgmat[t][t], M1 = C.dgmat[t][1 - t];
  const long cells_per_block = blockDim.x / NP;
  // persistent: blocks stride over the cells; the loop bound is uniform in
  // the block so every lane takes part in the warp-level exchanges
  for (long base = blockIdx.x * cells_per_block; base < ncb;
       base += (long)gridDim.x * cells_per_block) {
    long c = base + threadIdx.x / NP;
    bool valid = c < ncb;
    long cc = valid ? c : 0;
    bool active = valid && (mask == nullptr || mask[cc]);
    double flag = active ? qh[cc * NP * V] : 0.0;  // NaN sentinel of the Picard pass
    active = active && (flag != flag);
    if (__all_sync(0xffffffffu, !active))
      continue;
    const int inst = BATCH ? B.inst_b[cc] : 0;
    const DevPar &P = BATCH ? B.P[inst] : Pv;
    const double dt = BATCH ? B.clk[5 * inst + 1] : dt_in;
    const double idx = BATCH ? B.idx[inst] : idx_in;
    const double a_t = dt * C.w[t];
    double Ww[V], q[V], r[V], other[V];
    const double *wc = wh + (cc * NS + sidx) * V;
#pragma unroll
    for (int k = 0; k < V; k++) {
      double w = active ? wc[k] : 1.0;
      Ww[k] = f * w;
      q[k] = w;
    }
    bool done = !active;
    bool ok = false;
    int iters = 0;
    for (int it = 0; it < C.stiff_it; it++) {
      if (__all_sync(0xffffffffu, done))
        break;
      dg_rhs_node<L, ND>(q, Ww, r, t, i, j, dt, idx, idy, P, C);
      // residual g = r - W_s sum_m DG_MAT[t][m] q(m)
      shfl_vec<V>(q, other, TB);
#pragma unroll
      for (int k = 0; k < V; k++)
        r[k] -= ws * (M0 * q[k] + M1 * other[k]);
      if (!done) {
        Prim<L::THERMAL> st;
        prim<L::THERMAL>(q, P, st);
        // this time node's diagonal block A_t = M_tt I - a_t dS/dA of the
        // 18 x 18 Newton matrix (the off-diagonal blocks are M_t,1-t I) and
        // its right-hand side
        stiff_jacobian_rows<L::THERMAL>(q, st, P, a_t, M0, Am + t * 9 * NA + t * 9, NA,
                                        Jm + t * 3 * NJ + t * 3, NJ);
#pragma unroll
        for (int a = 0; a < 9; a++)
          Ab[t * 9 + a] = (float)(r[5 + a] * iws);
        if (L::THERMAL) {
#pragma unroll
          for (int a = 0; a < 3; a++)
            Jb[t * 3 + a] = (float)(r[14 + a] * iws);
        }
      }
      __syncwarp();
      // Block elimination of [[A0, m01 I], [m10 I, A1]] [x0; x1] = [b0; b1]:
      // (A0 A1 - m01 m10 I) x1 = A0 b1 - m10 b0 and x0 = (b1 - A1 x1) / m10,
      // a 9 x 9 solve (3 x 3 for the heat flux) in place of 18 x 18 (6 x 6).
      // The two time-node lanes form the reduced matrix's rows (into block
      // (0, 1) of Am), lane t = 0 its right-hand side (block (1, 0)'s first
      // row) and lane t = 1 the heat-flux system.
      const float m01 = (float)C.dgmat[0][1], m10 = (float)C.dgmat[1][0];
      const float *A0 = Am, *A1 = Am + 9 * NA + 9;
      float *Rm = Am + 9, *Rb = Am + 9 * NA;
      const float *J0 = Jm, *J1 = Jm + 3 * NJ + 3;
      float *RJm = Jm + 3, *RJb = Jm + 3 * NJ;
      if (!done) {
        const int r0 = t == 0 ? 0 : 5, r1 = t == 0 ? 5 : 9;
        for (int rr = r0; rr < r1; rr++) {
#pragma unroll
          for (int c = 0; c < 9; c++) {
            float acc = rr == c ? -m01 * m10 : 0.0f;
#pragma unroll
            for (int k = 0; k < 9; k++)
              acc = fmaf(A0[rr * NA + k], A1[k * NA + c], acc);
            Rm[rr * NA + c] = acc;
          }
        }
        if (t == 0) {
#pragma unroll
          for (int rr = 0; rr < 9; rr++) {
            float acc = -m10 * Ab[rr];
#pragma unroll
            for (int k = 0; k < 9; k++)
              acc = fmaf(A0[rr * NA + k], Ab[9 + k], acc);
            Rb[rr] = acc;
          }
        } else if (L::THERMAL) {
#pragma unroll
          for (int rr = 0; rr < 3; rr++) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
              float acc = rr == c ? -m01 * m10 : 0.0f;
#pragma unroll
              for (int k = 0; k < 3; k++)
                acc = fmaf(J0[rr * NJ + k], J1[k * NJ + c], acc);
              RJm[rr * NJ + c] = acc;
            }
            float acc = -m10 * Jb[rr];
#pragma unroll
            for (int k = 0; k < 3; k++)
              acc = fmaf(J0[rr * NJ + k], Jb[3 + k], acc);
            RJb[rr] = acc;
          }
        }
      }
      __syncwarp();
      bool solved = true;
      if (!done) {
        if (t == 0)
          solved = smem_solve<9>(Rm, NA, Rb);
        else if (L::THERMAL)
          solved = smem_solve<3>(RJm, NJ, RJb);
      }
      __syncwarp();
      // non-stiff variables: DG_MAT^-1 g / W_s (partner time node's residual)
      shfl_vec<V>(r, other, TB);
      double delta[V];
      double ia = C.dgmatinv[t][t] * iws, ib = C.dgmatinv[t][1 - t] * iws;
#pragma unroll
      for (int k = 0; k < V; k++)
        delta[k] = ia * r[k] + ib * other[k];
      // stiff variables: x1 from the reduced solve, x0 = (b1 - A1 x1) / m10
      const float im10 = 1.0f / m10;
#pragma unroll
      for (int a = 0; a < 9; a++) {
        float x = Rb[a];
        if (t == 0) {
          float acc = Ab[9 + a];
#pragma unroll
          for (int k = 0; k < 9; k++)
            acc = fmaf(-A1[a * NA + k], Rb[k], acc);
          x = acc * im10;
        }
        delta[5 + a] = (double)x;
      }
      if (L::THERMAL) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
          float x = RJb[a];
          if (t == 0) {
            float acc = Jb[3 + a];
#pragma unroll
            for (int k = 0; k < 3; k++)
              acc = fmaf(-J1[a * NJ + k], RJb[k], acc);
            x = acc * im10;
          }
          delta[14 + a] = (double)x;
        }
      }
      __syncwarp();
      bool big = false, bad = !solved;
#pragma unroll
      for (int k = 0; k < V; k++) {
        double qn = q[k] + delta[k];
        if (fabs(delta[k]) > C.stiff_tol * (1.0 + fabs(qn)))
          big = true;
        if (qn != qn)
          bad = true;
        if (!done)
          q[k] = qn;
      }
      unsigned bigm = __ballot_sync(0xffffffffu, big) & gmask;
      unsigned badm = __ballot_sync(0xffffffffu, bad) & gmask;
      if (!done) {
        iters = it + 1;
        if (badm) {
          done = true;
        } else if (!bigm) {
          done = true;
          ok = true;
        }
      }
    }
    if (active) {
      double *out = qh + (cc * NP + g) * V;
#pragma unroll
      for (int k = 0; k < V; k++)
        out[k] = q[k];
      if (status && g == 0)
        status[cc] = (ok ? GPR_PRED_NEWTON : GPR_PRED_FAILED) | (iters << 8);
    }
  }
}

// ---------------------------------------------------------------------------
// Finite-volume update (solvers/fv/fv.cpp:11-297).
//
// Face pass: one thread per (face, time node t[, transverse node s]).  It
// extrapolates qL, qR to the face, evaluates the Rusanov dissipation
// D = max(lambda_L, lambda_R)(qL - qR) + F(qL) + F(qR) (fluxes.cpp:66-75) and
// the path integral Bint (fluxes.cpp:9-20), weights them, and the NQ lanes
// of a face reduce with shuffles.  Face results: fb[face][0][k] (to the left
// cell, subtracted) and fb[face][1][k] (to the right cell).

template <class L>
GPR_D void interface_point(const double *ql, const double *qr, int d, const DevPar &P,
                           const Consts &C, double *f, double *b) {
  constexpr int V = L::V;
  Prim<L::THERMAL> sl, sr;
  prim<L::THERMAL>(ql, P, sl);
  prim<L::THERMAL>(qr, P, sr);
  double m1 = max_abs_eigs<L::THERMAL>(ql, sl, d, P);
  double m2 = max_abs_eigs<L::THERMAL>(qr, sr, d, P);
  double m = m1 > m2 ? m1 : m2;  // std::max(m1, m2)
#pragma unroll
  for (int k = 0; k < V; k++)
    f[k] = m * (ql[k] - qr[k]);
  flux_add<L::THERMAL, V>(ql, sl, d, P, f);
  flux_add<L::THERMAL, V>(qr, sr, d, P, f);
  // Bint: sum_i W_i B(qL + x_i dq) dq, dq = qR - qL; B needs only v
  double dq[V];
#pragma unroll
  for (int k = 0; k < V; k++) {
    dq[k] = qr[k] - ql[k];
    b[k] = 0.0;
  }
#pragma unroll
  for (int n = 0; n < NN; n++) {
    double rho = ql[0] + C.nodes[n] * dq[0];
    double ir = 1.0 / rho;
    double v[3] = {(ql[2] + C.nodes[n] * dq[2]) * ir, (ql[3] + C.nodes[n] * dq[3]) * ir,
                   (ql[4] + C.nodes[n] * dq[4]) * ir};
    double bd[V];
    bdot<V, L::LSET>(v, dq, d, bd);
#pragma unroll
    for (int k = 5; k < V; k++)  // B x is zero outside the distortion and level-set rows
      if (k < 14 || k >= V - L::LSET)
        b[k] += C.w[n] * bd[k];
  }
}

// 1D faces i = 0..nx between predictor cells i and i+1.  NQ = N lanes per
// face (time nodes).
template <class L, bool BATCH = false>
__global__ void __launch_bounds__(128) k_faces1d(
    double *__restrict__ fb, const double *__restrict__ qh, long nface,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    int time_dg, DevPar Pv, Consts C, Batch B) {
  constexpr int V = L::V;
  constexpr int NQ = NN;
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int t = threadIdx.x % NQ;
  long face = gt / NQ;
  bool valid = face < nface;
  long fo = valid ? face : 0;
  // predictor cell on the left of the face (packed index in the batched form)
  long fi = fo;
  const int inst = BATCH ? B.inst_f[fo] : 0;
  const DevPar &P = BATCH ? B.P[inst] : Pv;
  if (BATCH) {
    fi = B.off_b[inst] + (fo - B.off_f[inst]);
    dt = B.clk[5 * inst + 1];
    dx = 1.0 / B.idx[inst];
  }
  bool active = valid && (mask == nullptr || (mask[fi] && mask[fi + 1])) && (time_dg || t == 0);
  int nt = time_dg ? NN : 1;
  double ql[V], qr[V], f[V], b[V];
  const double *ql_ = qh + (fi * nt + (time_dg ? t : 0)) * NN * V;
  const double *qr_ = qh + ((fi + 1) * nt + (time_dg ? t : 0)) * NN * V;
#pragma unroll
  for (int k = 0; k < V; k++) {
    ql[k] = C.endv[1][0] * ql_[k] + C.endv[1][1] * ql_[V + k];
    qr[k] = C.endv[0][0] * qr_[k] + C.endv[0][1] * qr_[V + k];
  }
  double kk = (time_dg ? dt * C.w[t] : dt) / (2.0 * dx);
  if (active) {
    interface_point<L>(ql, qr, 0, P, C, f, b);
  } else {
#pragma unroll
    for (int k = 0; k < V; k++)
      f[k] = b[k] = 0.0;
  }
  face_reduce_store<V, NN>(b, f, kk, active, valid, t, fb + fo * 2 * V);
}

// 1D faces for small grids, where a kernel's time is the length of one
// lane's FP64 instruction chain: one lane per (face, time node, side).  The
// lane of side 0 (1) evaluates the primitives, wave speed and flux of qL
// (qR) and the path integral's node 0 (1); the wave speeds are exchanged,
// the side-0 lane adds the dissipation, and the four lanes' contributions
// are summed by the reduce-scatter (the same terms as interface_point).
template <class L, bool BATCH>
GPR_D void faces1d_split_body(double *__restrict__ fb, const double *__restrict__ qh,
                              long nface, const uint8_t *__restrict__ mask, double dt,
                              double dx, int time_dg, const DevPar &Pv, const Consts &C,
                              const Batch &B, long face, int lq, bool inrange, long fbase) {
  constexpr int V = L::V;
  static_assert(NN == 2, "two time nodes and two path nodes");
  const int t = lq >> 1, side = lq & 1;
  bool valid = inrange && face < nface;
  const long fo = valid ? face : 0;
  // predictor cell on the left of the face (packed index in the batched form)
  long fi = fo;
  const int inst = BATCH ? B.inst_f[fo] : 0;
  const DevPar &P = BATCH ? B.P[inst] : Pv;
  if (BATCH) {
    fi = B.off_b[inst] + (fo - B.off_f[inst]);
    dt = B.clk[5 * inst + 1];
    dx = 1.0 / B.idx[inst];
  }
  bool active = valid && (mask == nullptr || (mask[fi] && mask[fi + 1])) && (time_dg || t == 0);
  int nt = time_dg ? NN : 1;
  double ql[V], qr[V], f[V], b[V], dq[V];
  const double *ql_ = qh + (fi * nt + (time_dg ? t : 0)) * NN * V;
  const double *qr_ = qh + ((fi + 1) * nt + (time_dg ? t : 0)) * NN * V;
#pragma unroll
  for (int k = 0; k < V; k++) {
    ql[k] = C.endv[1][0] * ql_[k] + C.endv[1][1] * ql_[V + k];
    qr[k] = C.endv[0][0] * qr_[k] + C.endv[0][1] * qr_[V + k];
    dq[k] = qr[k] - ql[k];
    b[k] = 0.0;
  }
  const double kk = (time_dg ? dt * C.w[t] : dt) / (2.0 * dx);
  const double *qs = side ? qr : ql;
  Prim<L::THERMAL> ps;
  prim<L::THERMAL>(qs, P, ps);
  const double lam = max_abs_eigs<L::THERMAL>(qs, ps, 0, P);
  const double lo = __shfl_xor_sync(0xffffffffu, lam, 1);
  const double m1 = side ? lo : lam, m2 = side ? lam : lo;  // lambda(qL), lambda(qR)
  const double m = m1 > m2 ? m1 : m2;                        // std::max(m1, m2)
  flux_set<L::THERMAL, V>(qs, ps, 0, P, f);
  if (side == 0) {
#pragma unroll
    for (int k = 0; k < V; k++)
      f[k] += m * (ql[k] - qr[k]);
  }
  // Bint node `side`: W_n B(qL + x_n dq) dq   (fluxes.cpp:9-20)
  {
    const double xn = C.nodes[side], wn = C.w[side];
    double ir = 1.0 / (ql[0] + xn * dq[0]);
    double v[3] = {(ql[2] + xn * dq[2]) * ir, (ql[3] + xn * dq[3]) * ir,
                   (ql[4] + xn * dq[4]) * ir};
    double bd[V];
    bdot<V, L::LSET>(v, dq, 0, bd);
#pragma unroll
    for (int k = 5; k < V; k++)
      if (k < 14 || k >= V - L::LSET)
        b[k] = wn * bd[k];
  }
  face_reduce_store<V, 4>(b, f, kk, active, valid, lq, fb + (fo - fbase) * 2 * V);
}

template <class L, bool BATCH = false>
__global__ void __launch_bounds__(128) k_faces1d_split(
    double *__restrict__ fb, const double *__restrict__ qh, long nface,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    int time_dg, DevPar Pv, Consts C, Batch B) {
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  faces1d_split_body<L, BATCH>(fb, qh, nface, mask, dt, dx, time_dg, Pv, C, B, gt / 4,
                               threadIdx.x % 4, true, 0);
}

// 2D faces: direction dir, faces (i, j) of the (nx+1) x (ny+1) face grid,
// between predictor cells (i, j) and (i+1, j) (dir 0) or (i, j+1) (dir 1);
// NQ = N*N lanes per face (time node t, transverse node s).  parity < 0:
// every face, contributions written to fb[face][2][V] (the face-flux
// entry points); parity 0 / 1: the faces of that parity along dir, applied
// to u (passed as fb) in place, the conservative update of interfs2.
template <class L>
__global__ void __launch_bounds__(128) k_faces2d(
    double *__restrict__ fb, const double *__restrict__ qh, int nx, int ny, int dir,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    double dy, int time_dg, DevPar P, Consts C, int parity = -1) {
  constexpr int V = L::V;
  constexpr int NQ = NN * NN;
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int lq = threadIdx.x % NQ;
  int t = lq / NN, s = lq % NN;
  const Face2 F = face2_of(gt / NQ, nx, ny, dir, parity);
  const bool valid = F.valid;
  const long fi = F.fi;
  const int i = F.i, j = F.j;
  long cb = (long)i * (ny + 2) + j;
  long cn = dir == 0 ? cb + (ny + 2) : cb + 1;
  bool geo = dir == 0 ? (j > 0) : (i > 0);
  const bool face_on = valid && geo && (mask == nullptr || (mask[cb] && mask[cn]));
  bool active = face_on && (time_dg || t == 0);
  int nt = time_dg ? NN : 1;
  int tt = time_dg ? t : 0;
  const double *q0 = qh + (cb * nt + tt) * NN * NN * V;
  const double *q1 = qh + (cn * nt + tt) * NN * NN * V;
  double ql[V], qr[V], f[V], b[V];
  // endpts2d (evaluations.cpp:20-35): dir 0 -> nodes (m, s); dir 1 -> (s, m)
  long o0 = dir == 0 ? (long)s * V : (long)s * NN * V;
  long st = dir == 0 ? (long)NN * V : (long)V;
#pragma unroll
  for (int k = 0; k < V; k++) {
    ql[k] = C.endv[1][0] * q0[o0 + k] + C.endv[1][1] * q0[o0 + st + k];
    qr[k] = C.endv[0][0] * q1[o0 + k] + C.endv[0][1] * q1[o0 + st + k];
  }
  double wt = time_dg ? dt * C.w[t] : dt;
  double kk = wt / (2.0 * (dir == 0 ? dx : dy)) * C.w[s];
  if (active) {
    interface_point<L>(ql, qr, dir, P, C, f, b);
  } else {
#pragma unroll
    for (int k = 0; k < V; k++)
      f[k] = b[k] = 0.0;
  }
  if (parity < 0) {
    face_reduce_store<V, NQ>(b, f, kk, active, valid, lq, fb + fi * 2 * V);
  } else {
    double *uL, *uR;
    face2_cells(fb, i, j, nx, ny, dir, V, uL, uR);
    face_reduce_apply<V, NQ>(b, f, kk, active, face_on, lq, uL, uR);
  }
}

// Parts of the FV update k_cells applies: the volume term (centers1 /
// centers2, fv.cpp:11-109) and the face contributions (interfs1 / interfs2,
// fv.cpp:111-279); fv_launcher applies both.
constexpr int FV_CENTERS = 1, FV_INTERFS = 2, FV_BOTH = 3;

// Cell pass: one thread per (cell, space-time node): the volume term
// w_t w_s (S - B dq/dx [- B dq/dy]) (fv.cpp:11-109), reduced over the cell's
// NP lanes, then u += volume - face contributions (the parts selected).
// The body for cell c (u index), lane g of its NP lanes; fbx[(fo - fbase)]
// holds the 1D face on the cell's left (fbase: the first face of a tile
// staged in shared memory, else 0).
template <class L, int ND, bool BATCH>
GPR_D void cells_body(double *__restrict__ u, const double *__restrict__ qh,
                      const double *__restrict__ fbx, const double *__restrict__ fby, long nx,
                      int ny, const uint8_t *__restrict__ mask, double dt, double dx,
                      double dy, int sources, int time_dg, const DevPar &Pv, const Consts &C,
                      const Batch &B, int parts, long c, int g, bool inrange, long fbase) {
  constexpr int V = L::V;
  constexpr int NS = ND == 1 ? NN : NN * NN;
  constexpr int NP = NN * NS;
  constexpr int XB = ND == 1 ? 1 : 2;
  constexpr int YB = 1;
  long ncell = ND == 1 ? nx : (long)nx * ny;
  bool valid = inrange && c < ncell;
  long cc = valid ? c : 0;
  const int inst = BATCH ? B.inst_u[cc] : 0;
  const DevPar &P = BATCH ? B.P[inst] : Pv;
  double idx = 1.0 / dx;
  const double idy = 1.0 / dy;
  long ci = ND == 1 ? cc : (cc / ny);
  int cj = ND == 1 ? 0 : (int)(cc % ny);
  long cb = ND == 1 ? ci + 1 : (long)(ci + 1) * (ny + 2) + (cj + 1);
  long fo = ci;  // face on the left of the cell (1D)
  if (BATCH) {
    long li = cc - B.off_u[inst];
    cb = B.off_b[inst] + li + 1;
    fo = B.off_f[inst] + li;
    dt = B.clk[5 * inst + 1];
    idx = B.idx[inst];
  }
  bool active = valid && (mask == nullptr || mask[cb]);
  int t = g / NS, sidx = g % NS;
  int i = ND == 1 ? sidx : sidx / NN, j = ND == 1 ? 0 : sidx % NN;
  int nt = time_dg ? NN : 1;
  bool live = active && (time_dg || t == 0);
  int tt = time_dg ? t : 0;
  const double *qc = qh + ((cb * nt + tt) * NS + sidx) * V;
  double q[V], other[V], dq[V], acc[V];
#pragma unroll
  for (int k = 0; k < V; k++)
    acc[k] = 0.0;
  if (parts & FV_CENTERS) {
#pragma unroll
    for (int k = 0; k < V; k++)
      q[k] = qc[k];
    Prim<L::THERMAL> s;
    prim<L::THERMAL>(q, P, s);
    // wn (S - B dq/dx [- B dq/dy]), wn folded into the source's scalar
    // factors and the derivative coefficients (B is linear)
    const double wt = time_dg ? dt * C.w[t] : dt;
    const double wn = ND == 1 ? wt * C.w[i] : wt * C.w[i] * C.w[j];
    if (sources)
      source<L::THERMAL, V>(q, s, P, acc, wn);
    shfl_vec<V>(q, other, XB);
    {
      double a = C.derv[i][i] * idx * wn, b = C.derv[i][1 - i] * idx * wn;
#pragma unroll
      for (int k = 0; k < V; k++)
        dq[k] = a * q[k] + b * other[k];
      double bd[V];
      bdot<V, L::LSET>(s.v, dq, 0, bd);
#pragma unroll
      for (int k = 0; k < V; k++)
        acc[k] -= bd[k];
    }
    if (ND == 2) {
      shfl_vec<V>(q, other, YB);
      double a = C.derv[j][j] * idy * wn, b = C.derv[j][1 - j] * idy * wn;
#pragma unroll
      for (int k = 0; k < V; k++)
        dq[k] = a * q[k] + b * other[k];
      double bd[V];
      bdot<V, L::LSET>(s.v, dq, 1, bd);
#pragma unroll
      for (int k = 0; k < V; k++)
        acc[k] -= bd[k];
    }
#pragma unroll
    for (int k = 0; k < V; k++)
      acc[k] = live ? acc[k] : 0.0;
  }
  // the cell's sum over its NP lanes, scattered: lane g holds variables
  // g CK .. g CK + CK - 1
  constexpr int CK = (V + NP - 1) / NP;
  double red[CK * NP];
#pragma unroll
  for (int k = 0; k < CK * NP; k++)
    red[k] = k < V ? acc[k] : 0.0;
  if (parts & FV_CENTERS)
    GroupReduceScatter<CK * NP, NP>::run(red, g);
  else {
#pragma unroll
    for (int k = 0; k < CK; k++)
      red[k] = 0.0;
  }
  if (!valid || !active)
    return;
  const bool faces = parts & FV_INTERFS;
  double *uc = u + cc * V;
  if (ND == 1) {
    // face ci: R part, face ci+1: L part (fv.cpp:143-146)
    const double *fl = fbx + (fo - fbase) * 2 * V;
    const double *fr = fbx + (fo - fbase + 1) * 2 * V;
    bool okl = mask == nullptr || (mask[cb - 1] && mask[cb]);
    bool okr = mask == nullptr || (mask[cb] && mask[cb + 1]);
#pragma unroll
    for (int p = 0; p < CK; p++) {
      const int k = g * CK + p;
      if (k >= V)
        break;
      double x = uc[k] + red[p];
      if (faces && okr)
        x -= fr[k];
      if (faces && okl)
        x -= fl[V + k];
      uc[k] = x;
    }
  } else {
    // x faces (fi, fj) with fi = ci+1 (L part) and fi = ci (R part), fj = cj+1;
    // y faces fi = ci+1 with fj = cj+1 (L part) and fj = cj (R part).
    long fxl = (long)(ci + 1) * (ny + 1) + (cj + 1);  // L part to this cell
    long fxr = (long)ci * (ny + 1) + (cj + 1);        // R part to this cell
    long fyl = (long)(ci + 1) * (ny + 1) + (cj + 1);
    long fyr = (long)(ci + 1) * (ny + 1) + cj;
#pragma unroll
    for (int p = 0; p < CK; p++) {
      const int k = g * CK + p;
      if (k >= V)
        break;
      double x = uc[k] + red[p];
      if (faces) {
        x -= fbx[fxl * 2 * V + k];
        x -= fbx[fxr * 2 * V + V + k];
        x -= fby[fyl * 2 * V + k];
        x -= fby[fyr * 2 * V + V + k];
      }
      uc[k] = x;
    }
  }
}

template <class L, int ND, bool BATCH = false>
__global__ void __launch_bounds__(128) k_cells(
    double *__restrict__ u, const double *__restrict__ qh, const double *__restrict__ fbx,
    const double *__restrict__ fby, long nx, int ny, const uint8_t *__restrict__ mask,
    double dt, const double *__restrict__ dt_dev, double dx, double dy, int sources,
    int time_dg, DevPar Pv, Consts C, Batch B, int parts) {
  constexpr int NP = NN * (ND == 1 ? NN : NN * NN);
  if (dt_dev)
    dt = *dt_dev;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  cells_body<L, ND, BATCH>(u, qh, fbx, fby, nx, ny, mask, dt, dx, dy, sources, time_dg, Pv, C,
                           B, parts, gt / NP, threadIdx.x % NP, true, 0);
}

// The whole 1D FV update of fv_launcher (centers1 + interfs1, fv.cpp:11-160)
// in one launch, Rusanov flux: a block takes a tile of TILE cells; its
// 4 (TILE + 1) threads first evaluate the tile's TILE + 1 faces (one lane per
// face, time node and side, as k_faces1d_split) into shared memory, then
// the cells' volume terms (one lane per space-time node, as k_cells), and
// each cell's lanes apply u += volume - its two faces' contributions.  A
// face between two tiles is evaluated by both (one face in TILE + 1 twice);
// the sums and their order are those of the two-launch form.
// A small grid takes tiles of FV1_TILE_SMALL cells (one warp per block), so
// that its few warps run on separate SMs.
constexpr int FV1_TILE = 31;
constexpr int FV1_TILE_SMALL = 7;
template <class L, int TILE = FV1_TILE>
__global__ void __launch_bounds__(128) k_fv1d(
    double *__restrict__ u, const double *__restrict__ qh, long nx,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    int sources, int time_dg, DevPar P, Consts C, int parts) {
  constexpr int V = L::V;
  static_assert(NN == 2 && 4 * (TILE + 1) <= 128 && (TILE + 1) % 8 == 0,
                "four lanes per face and per cell, whole warps");
  __shared__ double sfb[(TILE + 1) * 2 * V];
  if (dt_dev)
    dt = *dt_dev;
  const long c0 = (long)blockIdx.x * TILE;  // first cell, and first face, of the tile
  const int slot = threadIdx.x >> 2, lq = threadIdx.x & 3;
  if (parts & FV_INTERFS)
    faces1d_split_body<L, false>(sfb, qh, nx + 1, mask, dt, dx, time_dg, P, C, Batch{},
                                 c0 + slot, lq, true, c0);
  __syncthreads();
  cells_body<L, 1, false>(u, qh, sfb, nullptr, nx, 1, mask, dt, dx, 1.0, sources, time_dg, P, C,
                          Batch{}, parts, c0 + slot, lq, slot < TILE, c0);
}

// ---------------------------------------------------------------------------
// CFL time step (solvers/iterator.cpp:54-83): per-cell sum_d mae/dx_d,
// block max, atomicMax on the bit pattern (non-negative doubles order as
// unsigned integers); NaN cells are skipped as std::max skips them.
template <class L>
__global__ void __launch_bounds__(256) k_cfl_max(const double *__restrict__ u, long ncell,
                                                 int nd, double dx, double dy,
                                                 unsigned long long *__restrict__ out,
                                                 DevPar P) {
  constexpr int V = L::V;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  double m = 0.0;
  if (c < ncell) {
    double q[V];
#pragma unroll
    for (int k = 0; k < V; k++)
      q[k] = u[c * V + k];
    Prim<L::THERMAL> s;
    prim<L::THERMAL>(q, P, s);
    double tmp = max_abs_eigs<L::THERMAL>(q, s, 0, P) / dx;
    if (nd == 2)
      tmp += max_abs_eigs<L::THERMAL>(q, s, 1, P) / dy;
    if (tmp > m)
      m = tmp;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0)
    sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
      b = fmax(b, sm[w]);
    atomicMax(out, (unsigned long long)__double_as_longlong(b));
  }
}

static __global__ void k_cfl_finalize(const unsigned long long *__restrict__ mx, double cfl, double t,
                               double tf, int count, double *__restrict__ dt_out) {
  double MAX = __longlong_as_double((long long)*mx);
  double dt = cfl / MAX;
  if (count <= 5)
    dt *= 0.2;
  if (t + dt > tf)
    dt = tf - t;
  *dt_out = dt;
}

// Device clock of the device-resident time loop: [t, dt, tf, cfl, count].
// The CFL finalize reads t/count and writes dt (0 once t >= tf); the advance
// kernel adds dt to t and counts the step.
// flag (optional): the step's contortion flag, cleared here for the
// contortion check later in the same step.
static __global__ void k_clock_finalize(const unsigned long long *__restrict__ mx,
                                        double *__restrict__ clk, int *__restrict__ flag = nullptr) {
  if (flag)
    *flag = 0;
  double t = clk[0], tf = clk[2], cfl = clk[3];
  long count = (long)clk[4];
  double dt = 0.0;
  if (t < tf) {
    double MAX = __longlong_as_double((long long)*mx);
    dt = cfl / MAX;
    if (count <= 5)
      dt *= 0.2;
    if (t + dt > tf)
      dt = tf - t;
  }
  clk[1] = dt;
}

// mx (optional): the CFL maximum, cleared here for the next step's k_cfl_max.
static __global__ void k_clock_advance(double *__restrict__ clk,
                                       unsigned long long *__restrict__ mx = nullptr) {
  if (clk[1] > 0.0) {
    clk[0] += clk[1];
    clk[4] += 1.0;
  }
  if (mx)
    *mx = 0ull;
}

// renorm_distortion (solvers/utils.cpp:6-23); skipped when the device clock
// says the step did not run (dt == 0).
template <int V>
__global__ void k_renorm(double *__restrict__ u, long ncell, double rho0,
                         const double *__restrict__ dt_dev) {
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  if (dt_dev && *dt_dev == 0.0)
    return;
  double *q = u + c * V;
  double r = q[0];
  if (r > 0) {
    double A[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
      A[k] = q[5 + k];
    double f = cbrt(r / (rho0 * det3(A)));
#pragma unroll
    for (int k = 0; k < 9; k++)
      q[5 + k] = A[k] * f;
  }
}

// k_renorm followed by the contortion test of the renormalised cell
// (contorted, solvers/utils.cpp:66-85, as k_contorted): one launch for both.
template <int V>
__global__ void k_renorm_contorted(double *__restrict__ u, long ncell, double rho0, double tol,
                                   int *__restrict__ flag, const double *__restrict__ dt_dev) {
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  if (dt_dev && *dt_dev == 0.0)
    return;
  double *q = u + c * V;
  double A[9];
#pragma unroll
  for (int k = 0; k < 9; k++)
    A[k] = q[5 + k];
  const double r = q[0];
  if (r > 0) {
    double f = cbrt(r / (rho0 * det3(A)));
#pragma unroll
    for (int k = 0; k < 9; k++) {
      A[k] *= f;
      q[5 + k] = A[k];
    }
  }
  double f2 = 0.0;
#pragma unroll
  for (int k = 0; k < 9; k++)
    f2 += A[k] * A[k];
  double d13 = cbrt(fabs(det3(A)));
  if (f2 / (3.0 * d13 * d13) - 1.0 > tol)
    atomicOr(flag, 1);
}

// ---------------------------------------------------------------------------
// Batched helper kernels (1D).

// ub of every instance: interior copy and ghost cells (grid.cpp:12-125,
// 147-160), one thread per (packed ub cell, variable).
template <int V>
__global__ void k_b_boundaries(const double *__restrict__ u, double *__restrict__ ub,
                               long nub, Batch B) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= nub * V)
    return;
  int k = idx % V;
  long cb = idx / V;
  int inst = B.inst_ub[cb];
  int nx = B.nx[inst];
  long li = cb - B.off_ub[inst];
  const double *ui = u + (long)B.off_u[inst] * V;
  if (li >= NN && li < nx + NN) {
    ub[cb * V + k] = ui[(li - NN) * V + k];
    return;
  }
  int side = li >= nx + NN;
  int gi = side ? (int)(li - nx - NN) : (int)li;
  int code = B.bc[2 * inst + side];
  int si = bc_src_index(code, side, gi, nx);
  if (code == GPR_BC_PERIODIC)
    code = GPR_BC_TRANSMISSIVE;
  ub[cb * V + k] = bc_value<V>(code, 0, k, ui + (long)si * V);
}

// WENO per (packed predictor cell, variable)
template <int V>
__global__ void k_b_weno(double *__restrict__ wh, const double *__restrict__ ub, long ncb,
                         Consts C, Batch B) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= ncb * V)
    return;
  int k = idx % V;
  long c = idx / V;
  int inst = B.inst_b[c];
  long li = c - B.off_b[inst];
  const double *d0 = ub + ((long)B.off_ub[inst] + li) * V + k;
  weno_point(d0, V, wh + c * NN * V + k, V, (int)li, B.nx[inst] + 2, 0, C);
}

// per-instance CFL maximum: atomicMax of the bit pattern per instance
template <class L>
__global__ void __launch_bounds__(256) k_b_cfl_max(const double *__restrict__ u, long ncell,
                                                   unsigned long long *__restrict__ mx,
                                                   Batch B, double *__restrict__ mcell = nullptr) {
  constexpr int V = L::V;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  int inst = B.inst_u[c];
  const DevPar &P = B.P[inst];
  double q[V];
#pragma unroll
  for (int k = 0; k < V; k++)
    q[k] = u[c * V + k];
  Prim<L::THERMAL> s;
  prim<L::THERMAL>(q, P, s);
  double m = max_abs_eigs<L::THERMAL>(q, s, 0, P) * B.idx[inst];
  if (mcell)
    mcell[c] = m;
  if (m > 0.0)  // NaN and zero are skipped
    atomicMax(mx + inst, (unsigned long long)__double_as_longlong(m));
}

// per-instance dt (iterator.cpp:54-83 per instance) and the step counter
static __global__ void k_b_clock_finalize(unsigned long long *__restrict__ mx, Batch B) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B.ninst)
    return;
  double *c = B.clk + 5 * k;
  double t = c[0], tf = c[2], cfl = c[3];
  long count = (long)c[4];
  double dt = 0.0;
  if (t < tf) {
    double MAX = __longlong_as_double((long long)mx[k]);
    dt = cfl / MAX;
    if (count <= 5)
      dt *= 0.2;
    if (t + dt > tf)
      dt = tf - t;
  }
  c[1] = dt;
  mx[k] = 0ull;  // ready for the next step's maximum
}

template <int V>
__global__ void k_b_renorm(double *__restrict__ u, long ncell, Batch B) {
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  int inst = B.inst_u[c];
  if (B.clk[5 * inst + 1] == 0.0)
    return;
  double *q = u + c * V;
  double r = q[0];
  if (r > 0) {
    double A[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
      A[k] = q[5 + k];
    double f = cbrt(r / (B.P[inst].rho0 * det3(A)));
#pragma unroll
    for (int k = 0; k < 9; k++)
      q[5 + k] = A[k] * f;
  }
}

static __global__ void k_b_clock_advance(Batch B, unsigned long long *__restrict__ updates) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B.ninst)
    return;
  double *c = B.clk + 5 * k;
  if (c[1] > 0.0) {
    c[0] += c[1];
    c[4] += 1.0;
    if (updates)
      atomicAdd(updates, (unsigned long long)B.nx[k]);
  }
}

}  // namespace gpr
