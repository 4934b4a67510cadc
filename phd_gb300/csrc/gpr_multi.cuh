// gpr_multi.cuh - level-set ghost fluid on the device (one level set, at most
// two materials, no heat conduction: the V = 15 layout).
//
// Restates the reference's multi/ module and the interface Riemann problem
// it calls:
//   re-distancing        multi/pfmm.cpp:4-26 (first-order fast marching of
//                        the vendored scikit-fmm, distance_marcher.cpp,
//                        base_marcher.cpp)
//   normals              multi/functions.cpp:16-54 (finite_difference)
//   interface cells      multi/fill.cpp:20-74 (find_interface_cells)
//   boundary fill        multi/fill.cpp:96-235 (fill_boundary_cells)
//   layered fill         multi/fill.cpp:237-328 (fill_neighbor_cells)
//   star state           system/multi/riemann.cpp:26-233, conditions.cpp,
//                        rotations.cpp, functions/vectors.cpp:85-154
//   merge, CFL, renorm   solvers/iterator.cpp:12-83, solvers/utils.cpp:6-23
//
// The reference runs every piece as a sequential sweep over the grid.  Here
// each is a data-parallel kernel whose result equals the sequential sweep:
//   * the fast marching order is replaced by tiled sweeps of the same
//     causal upwind update, whose fixed point is what the marcher computes
//     (band neighbours always enter a point's quadratic, the others only
//     while their distance is below the point's estimate, as the marcher's
//     heap order makes it), in FP64 with the marcher's quadratic and
//     roundings;
//   * a boundary cell reads the right-hand state of the interface from a
//     cell that an earlier cell of the (i, j) sweep may have filled; those
//     reads are resolved to the last earlier writer and solved level by
//     level (almost every cell is on level 0);
//   * within one layer of the extrapolation, a cell copies from a cell of the
//     same layer only if the sweep reached that one first; that chain is
//     followed explicitly.
#pragma once

#include <float.h>

#include "gpr_kernels.cuh"
#include "gpr_ode.cuh"

namespace gpr {
namespace multi {

// Grid of nd = 1 (ny = 1) or 2 dimensions; cell (i, j) is flat index
// i * ny + j, the reference's cell order.
struct Grid {
  int nd, nx, ny;
  long ncell;
  double dx, dy;
};

// Non-contracted FP64 arithmetic where the result feeds a discontinuous
// decision (index truncation, marcher ordering): the same roundings as the
// reference's separate multiplies and adds.
GPR_D double mul(double a, double b) { return __dmul_rn(a, b); }
GPR_D double add(double a, double b) { return __dadd_rn(a, b); }
GPR_D double sub(double a, double b) { return __dsub_rn(a, b); }
GPR_D double dvd(double a, double b) { return __ddiv_rn(a, b); }

// ===========================================================================
// Re-distancing (first-order fast marching, no narrow band, not periodic).

// Frozen band (initalizeFrozen, distance_marcher.cpp:90-151, with the
// reference's edit: the least per-axis crossing distance): cells where phi
// is zero or changes sign across a face, in FP64 with the marcher's
// roundings.  Others start unknown (+inf).  phi[c * ps] is the level set of
// cell c.  fz: bit 0 frozen (band), bit 1 the marcher would take the
// positive root for this cell (phi > DBL_EPSILON), bit 2 the point waits
// for an update (set by the sweeps); par: the neighbours that entered the
// point's update (set by the sweeps).
__global__ void k_fmm_init(const double *__restrict__ phi, long ps, double *__restrict__ d,
                           uint8_t *__restrict__ fz, uint8_t *__restrict__ par, Grid g,
                           int *__restrict__ anyfrozen, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= g.ncell)
    return;
  int i = g.nd == 1 ? (int)c : (int)(c / g.ny), j = g.nd == 1 ? 0 : (int)(c % g.ny);
  double p = phi[c * ps];
  uint8_t pos = p > DBL_EPSILON ? 2 : 0;
  double x = INFINITY;
  bool frozen = false;
  if (p == 0.0) {
    x = 0.0;
    frozen = true;
  } else {
    double ld[2] = {0.0, 0.0};
    bool borders = false;
    for (int dim = 0; dim < g.nd; dim++) {
      double h = dim == 0 ? g.dx : g.dy;
      for (int dir = -1; dir < 2; dir += 2) {
        int ii = dim == 0 ? i + dir : i, jj = dim == 1 ? j + dir : j;
        if (ii < 0 || ii >= g.nx || jj < 0 || jj >= g.ny)
          continue;
        double pn = phi[((long)ii * g.ny + jj) * ps];
        if (mul(p, pn) < 0.0) {
          borders = true;
          double dd = dvd(mul(h, p), sub(p, pn));
          if (ld[dim] == 0.0 || ld[dim] > dd)
            ld[dim] = dd;
        }
      }
    }
    if (borders) {
      double m = DBL_MAX;
      for (int dim = 0; dim < g.nd; dim++) {
        double t = fabs(ld[dim]);
        if (t > 0.0)
          m = t < m ? t : m;
      }
      x = p < 0.0 ? -m : m;
      frozen = true;
    }
  }
  d[c] = x;
  fz[c] = (frozen ? 1 : 0) | pos;
  par[c] = 0;
  if (frozen)
    atomicOr(anyfrozen, 1);
}

// Grid constants of the update: the marcher's idx2 = 1 / dx^2, 1 / dy^2
// (distance_marcher.cpp), its quadratic's leading coefficient for each set
// of entered axes (idx2[0], idx2[1], idx2[0] + idx2[1], as the marcher sums
// it) and that coefficient's reciprocal rounded to nearest, and the
// spacings.
struct FmmConst {
  double idx2[2], a[3], a4[3], ra[3], h[2], ih[2];
};

inline FmmConst fmm_const(double dx, double dy) {
  FmmConst K;
  K.idx2[0] = 1.0 / dx / dx;
  K.idx2[1] = 1.0 / dy / dy;
  K.a[0] = K.idx2[0];
  K.a[1] = K.idx2[1];
  K.a[2] = K.idx2[0] + K.idx2[1];
  for (int k = 0; k < 3; k++) {
    K.a4[k] = 4.0 * K.a[k];
    K.ra[k] = 1.0 / K.a[k];
  }
  K.h[0] = dx;
  K.h[1] = dy;
  K.ih[0] = 1.0 / dx;
  K.ih[1] = 1.0 / dy;
  return K;
}

// updatePointOrderOne + solveQuadratic (distance_marcher.cpp:5-28, 72-88)
// for the entered axes (use): a = sum idx2, b = -sum 2 idx2 v, c = sum idx2
// v^2 - 1, root (-b +- sqrt(b^2 - 4ac)) / 2 / a by the sign of phi, in FP64
// with the marcher's operation order and the fused multiply-adds of the
// reference's -O3 -march=native build (CMakeLists.txt:14): b and c
// accumulate by fma, det = fma(b, b, -(4 a c)); every other operation is
// rounded on its own.  The halving is a multiply by 0.5 (exact, the same
// value) and the division by a is Markstein's correction of a product with
// the rounded reciprocal, q = RN(q0 + RN(x - a q0) ra) with q0 = RN(x ra)
// (P. Markstein, IBM J. Res. Dev. 34, 1990; the correctly rounded quotient
// when ra = RN(1/a), as __ddiv_rn gives it).  The marcher leaves a point
// unchanged when the quadratic has no real root (its 0 return); so does a
// false return here.
GPR_D bool fmm_root(const double v[2], const bool use[2], const FmmConst &K, int nd, bool pos,
                    double &x) {
  // a (the sum of the entered idx2, in the marcher's order) and 4a are
  // tabulated per set of entered axes
  double b = 0.0, c = 0.0;
  for (int dim = 0; dim < nd; dim++)
    if (use[dim]) {
      b = __fma_rn(-mul(K.idx2[dim], 2.0), v[dim], b);
      c = __fma_rn(K.idx2[dim], mul(v[dim], v[dim]), c);
    }
  const int ka = use[0] && use[1] ? 2 : (use[0] ? 0 : 1);
  c = sub(c, 1.0);
  const double det = __fma_rn(b, b, -mul(K.a4[ka], c));
  if (!(det > 0.0))
    return false;
  const double sq = __dsqrt_rn(det);
  const double num = mul(pos ? add(-b, sq) : sub(-b, sq), 0.5);
  const double q0 = mul(num, K.ra[ka]);
  x = __fma_rn(__fma_rn(-q0, K.a[ka], num), K.ra[ka], q0);
  return x != 0.0;
}

// Update of one unfrozen point from its neighbours' current values
// (signed; +inf unknown), reproducing what the marcher's heap order makes
// of it (base_marcher.cpp:98-188): band neighbours (frozen at
// initialisation) always enter; the other neighbours enter in increasing
// |d| (equal keys together, as the marcher freezes them in one batch) while
// their |d| is below the point's current estimate, i.e. they were frozen
// before the point; after each entry the quadratic of the entered set is
// the new estimate, or, without a real root, the estimate stays (the
// marcher's 0 return).  Per axis the entered neighbour of least |d| is used
// (the lower one on ties, as the marcher scans -1 then +1).  Where
// rounding makes the new estimate fall below the neighbour that entered (a
// noise-level tie), the marcher keeps it and freezes the point next, so
// the point cannot enter that neighbour: each point records the
// non-band neighbours that entered it (mask bits 2 dim + side), and a
// neighbour that recorded this point is not a candidate here.  Returns
// `old` when nothing is known.
//
// A one-axis root is v +- h up to the quadratic's cancellation (at most
// ~eps (v^2 / h + |v| + h)); it is kept in that form while it only decides
// whether the next neighbour enters and the decision is clear by 256 times
// that bound, and evaluated exactly where it is the result or the decision
// is close.  The result is the same as evaluating every root exactly.
//
// |x| compares as the integer of its bits (the order of |x| for finite
// values and infinity), on the integer pipe.
GPR_D unsigned long long fmm_key(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

GPR_D double fmm_update(const double nb[2][2], const bool band[2][2], const bool excl[2][2],
                        bool pos, int nd, double old, const FmmConst &K, int &mask) {
  const double INF = INFINITY;
  const unsigned long long KINF = 0x7ff0000000000000ull;
  double v[2] = {INF, INF}, cv[2] = {INF, INF};
  unsigned long long ck[2] = {KINF, KINF};
  int cs[2] = {0, 0};
  bool use[2] = {false, false};
  for (int dim = 0; dim < nd; dim++)
    for (int s = 0; s < 2; s++) {
      const double x = nb[dim][s];
      const unsigned long long kx = fmm_key(x);
      if (band[dim][s]) {
        if (!use[dim] || kx < fmm_key(v[dim])) {
          v[dim] = x;
          use[dim] = true;
        }
      } else if (!excl[dim][s] && kx < ck[dim]) {
        ck[dim] = kx;
        cv[dim] = x;
        cs[dim] = s;
      }
    }
  mask = 0;
  double t = INF, tm = 0.0;  // tm > 0: t is v +- h, within tm of the exact root
  if (use[0] || use[1]) {
    double r;
    if (fmm_root(v, use, K, nd, pos, r))
      t = r;
  }
  bool done[2] = {ck[0] == KINF, nd < 2 || ck[1] == KINF};
  while (!done[0] || !done[1]) {
    const int a = done[0] ? 1 : (done[1] ? 0 : (ck[1] < ck[0] ? 1 : 0));
    const unsigned long long key = ck[a];
    if (tm > 0.0 && fabs(fabs(cv[a]) - fabs(t)) <= tm) {
      double r;
      if (fmm_root(v, use, K, nd, pos, r))
        t = r;
      tm = 0.0;
    }
    if (!(key < fmm_key(t)))
      break;
    const bool both = !done[1 - a] && ck[1 - a] == key;
    for (int q = 0; q < 2; q++) {
      const int dim = q == 0 ? a : 1 - a;
      if (q == 1 && !both)
        break;
      if (!use[dim] || fmm_key(cv[dim]) < fmm_key(v[dim])) {
        v[dim] = cv[dim];
        use[dim] = true;
      }
      mask |= 1 << (2 * dim + cs[dim]);
      done[dim] = true;
    }
    if (use[0] && use[1]) {
      double r;
      if (fmm_root(v, use, K, nd, pos, r)) {
        t = r;
        tm = 0.0;
      }
    } else {
      // v +- h of the one entered axis, and the bound of its distance from
      // the marcher's root
      const int k = use[0] ? 0 : 1;
      const double w = fabs(v[k]), h = K.h[k];
      const double t2 = pos ? v[k] + h : v[k] - h;
      const double m2 = 256.0 * DBL_EPSILON * (w * w * K.ih[k] + w + h);
      if (fabs(t2) > m2) {
        t = t2;
        tm = m2;
      } else {
        double r;
        if (fmm_root(v, use, K, nd, pos, r)) {
          t = r;
          tm = 0.0;
        }
      }
    }
  }
  if (tm > 0.0) {
    double r;
    if (fmm_root(v, use, K, nd, pos, r))
      t = r;
  }
  return isinf(t) ? old : t;
}

// The four neighbours of shared-memory point m (x neighbours m -+ o0, y
// neighbours m -+ 1) and whether each is in the frozen band.
template <int ND>
GPR_D void fmm_load_nb(const double *src, const uint8_t *sf, int m, int o0, double nb[2][2],
                       bool bd[2][2]) {
  nb[0][0] = src[m - o0];
  nb[0][1] = src[m + o0];
  bd[0][0] = sf[m - o0] & 1;
  bd[0][1] = sf[m + o0] & 1;
  if (ND == 2) {
    nb[1][0] = src[m - 1];
    nb[1][1] = src[m + 1];
    bd[1][0] = sf[m - 1] & 1;
    bd[1][1] = sf[m + 1] & 1;
  } else {
    nb[1][0] = nb[1][1] = INFINITY;
    bd[1][0] = bd[1][1] = false;
  }
}

// One round of tiled Jacobi sweeps of the causal update, in FP64.  Each
// block loads its tile and a one-cell halo into shared memory and runs up
// to `nsweeps` sweeps against that halo, then writes back.  A point waits
// for an update (dirty) when a neighbour changed after its last update;
// each sweep gathers the waiting points into a list first, so that whole
// warps run the updates, and a changed point makes its unfrozen tile
// neighbours wait.  GB300's FP64 pipe issues one warp instruction per 64
// cycles per SM partition, so the sweeps' cost is the longest chain of
// dependent updates (~1400 sweeps at 800 x 400, a tile crossed per round)
// times the update's FP64 instruction count, which the update above keeps
// to about one root.  The sweeps end when no point waits, at the fixed
// point of the update, whatever the order of the work.  lastg[c] is the
// round of cell c's last change; fz bit 2 carries a waiting point into the
// next round.  A tile runs if it has waiting points or a neighbouring tile
// changed in the previous round (tflag bit 1 / bit 0 of round - 1);
// flags[round] records whether anything changed or waits, and a round after
// a round without either returns at once.  2D tiles are 32 x 32 cells, 1D
// tiles 1024.  On the 800 x 400 shock bubble 8 x 8 tiles take the step
// from 23.8 to 22.5 ms against 16 x 16 ones: the front's tiles spread over
// more SMs, though the sweeps make more updates (33 per cell on the static
// circle, 91 after 13 steps of advection, against 34 and 60) along about
// the same chain of 1350-1650 dependent sweeps.  Each thread owns one 2D
// cell or two 1D cells.
constexpr int FMM_T2 = 8, FMM_T1 = 1024;
template <int ND> struct FmmThreads {
  static constexpr int value = ND == 2 ? 64 : 512;
};

template <int ND>
__global__ void __launch_bounds__(FmmThreads<ND>::value, ND == 2 ? 16 : 2)
    k_fmm_round(double *__restrict__ d, uint8_t *__restrict__ fz, uint8_t *__restrict__ par,
                int *__restrict__ lastg, Grid g, FmmConst K, int *__restrict__ flags, int *__restrict__ tflag, int round,
                int nsweeps, int mono, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  if (round > 0 && flags[round - 1] == 0)
    return;
  constexpr int TX = ND == 2 ? FMM_T2 : FMM_T1, TY = ND == 2 ? FMM_T2 : 1;
  constexpr int SX = TX + 2, SY = ND == 2 ? TY + 2 : 1;
  constexpr int FMM_THREADS = FmmThreads<ND>::value;
  constexpr int NT = TX * TY, PER = NT / FMM_THREADS, NW = FMM_THREADS / 32;
  const int ntx0 = (g.nx + TX - 1) / TX, nty0 = ND == 2 ? (g.ny + TY - 1) / TY : 1;
  const int ntiles = ntx0 * nty0;
  const int t = blockIdx.x;
  if (round > 0) {
    const int *prev = tflag + (long)(round - 1) * ntiles;
    int ti = ND == 2 ? t % ntx0 : t, tj = ND == 2 ? t / ntx0 : 0;
    bool run = prev[t] != 0 || (ti > 0 && (prev[t - 1] & 1)) ||
               (ti < ntx0 - 1 && (prev[t + 1] & 1)) ||
               (ND == 2 && ((tj > 0 && (prev[t - ntx0] & 1)) ||
                            (tj < nty0 - 1 && (prev[t + ntx0] & 1))));
    if (!run)
      return;
  }
  __shared__ double sd[SX * SY];
  __shared__ double nvs[NT];
  __shared__ uint8_t sf[SX * SY];
  __shared__ uint8_t sp[SX * SY];    // the neighbours that entered each point
  __shared__ uint8_t nms[NT];        // new masks of a sweep's updates
  __shared__ uint8_t hchg[SX * SY];  // halo point changed in the previous round
  __shared__ uint8_t dirty[NT];
  __shared__ uint8_t chg[NT];  // changed in this round
  __shared__ int16_t list[NT];
  __shared__ int wcnt[NW], total;
  const int bi = ND == 2 ? t % ntx0 : t, bj = ND == 2 ? t / ntx0 : 0;
  const int i0 = bi * TX, j0 = bj * TY;
  for (int e = threadIdx.x; e < SX * SY; e += FMM_THREADS) {
    int a = ND == 2 ? e / SY : e, b = ND == 2 ? e % SY : 0;
    int ii = i0 + a - 1, jj = ND == 2 ? j0 + b - 1 : 0;
    double x = INFINITY;
    uint8_t f = 0, hc = 0, pm = 0;
    if (ii >= 0 && ii < g.nx && jj >= 0 && jj < g.ny) {
      long c = (long)ii * g.ny + jj;
      x = d[c];
      f = fz[c];
      pm = par[c];
      hc = lastg[c] == round - 1;
    }
    sd[e] = x;
    sf[e] = f;
    sp[e] = pm;
    hchg[e] = hc;
  }
  auto smem_of = [&](int l) {
    return ND == 2 ? (l / TY + 1) * SY + (l % TY + 1) : l + 1;
  };
  auto inside_of = [&](int l) {
    int i = i0 + (ND == 2 ? l / TY : l), j = ND == 2 ? j0 + l % TY : 0;
    return i < g.nx && j < g.ny;
  };
  auto cell_of = [&](int l) {
    int i = i0 + (ND == 2 ? l / TY : l), j = ND == 2 ? j0 + l % TY : 0;
    return (long)i * g.ny + j;
  };
  auto is_halo = [&](int m) {
    int a = ND == 2 ? m / SY : m, b = ND == 2 ? m % SY : 1;
    return a == 0 || a == SX - 1 || (ND == 2 && (b == 0 || b == SY - 1));
  };
  const int o0 = ND == 2 ? SY : 1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  bool act[PER];
  for (int k = 0; k < PER; k++) {
    const int l = threadIdx.x + k * FMM_THREADS, m = smem_of(l);
    act[k] = inside_of(l) && !(sf[m] & 1);
    bool dd = act[k] && (round == 0 || (sf[m] & 4));
    if (act[k] && !dd) {
      const int nbm[4] = {m - o0, m + o0, m - 1, m + 1};
      for (int q = 0; q < (ND == 2 ? 4 : 2); q++)
        dd = dd || (is_halo(nbm[q]) && hchg[nbm[q]]);
    }
    dirty[l] = dd;
    chg[l] = 0;
  }
  __syncthreads();
  for (int it = 0; it < nsweeps; it++) {
    // 1. gather the waiting points (each thread clears its own flags)
    int mine = 0;
    bool sel[PER];
    for (int k = 0; k < PER; k++) {
      const int l = threadIdx.x + k * FMM_THREADS;
      sel[k] = dirty[l] != 0;
      dirty[l] = 0;
      mine += sel[k];
    }
    int incl = mine;  // inclusive warp scan
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o)
        incl += y;
    }
    if (lane == 31)
      wcnt[wid] = incl;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < wid; w++)
      base += wcnt[w];
    int pos = base + incl - mine;
    for (int k = 0; k < PER; k++)
      if (sel[k])
        list[pos++] = (int16_t)(threadIdx.x + k * FMM_THREADS);
    if (threadIdx.x == FMM_THREADS - 1)
      total = pos;
    __syncthreads();
    const int n = total;
    if (n == 0)
      break;
    // 2. updates (Jacobi: read the neighbours, write after a barrier)
    for (int q = threadIdx.x; q < n; q += FMM_THREADS) {
      const int m = smem_of(list[q]);
      double nb[2][2];
      bool bd[2][2];
      fmm_load_nb<ND>(sd, sf, m, o0, nb, bd);
      // a neighbour that recorded this point as entered (its bit for the
      // opposite side) is not a candidate
      bool ex[2][2];
      ex[0][0] = (sp[m - o0] >> 1) & 1;
      ex[0][1] = sp[m + o0] & 1;
      ex[1][0] = ND == 2 && ((sp[m - 1] >> 3) & 1);
      ex[1][1] = ND == 2 && ((sp[m + 1] >> 2) & 1);
      int msk;
      nvs[q] = fmm_update(nb, bd, ex, (sf[m] & 2) != 0, ND, sd[m], K, msk);
      nms[q] = (uint8_t)msk;
    }
    __syncthreads();
    // 3. take the new values (from the second half of the round budget on,
    // only a smaller |d|, which guarantees termination); the unfrozen tile
    // neighbours of a changed point wait for the next sweep
    for (int q = threadIdx.x; q < n; q += FMM_THREADS) {
      const int l = list[q], m = smem_of(l);
      const double old = sd[m], nv = nvs[q];
      if (mono ? fabs(nv) < fabs(old) : (nv != old || nms[q] != sp[m])) {
        sd[m] = nv;
        sp[m] = nms[q];
        chg[l] = 1;
        const int nbm[4] = {m - o0, m + o0, m - 1, m + 1};
        const int nbl[4] = {ND == 2 ? l - TY : l - 1, ND == 2 ? l + TY : l + 1, l - 1, l + 1};
        for (int k = 0; k < (ND == 2 ? 4 : 2); k++)
          if (!is_halo(nbm[k]) && !(sf[nbm[k]] & 1) && inside_of(nbl[k]))
            dirty[nbl[k]] = 1;
      }
    }
    __syncthreads();
  }
  bool wrote = false, waits = false;
  for (int k = 0; k < PER; k++) {
    const int l = threadIdx.x + k * FMM_THREADS;
    if (!act[k])
      continue;
    const int m = smem_of(l);
    const long c = cell_of(l);
    if (chg[l]) {
      d[c] = sd[m];
      par[c] = sp[m];
      lastg[c] = round;
      wrote = true;
    }
    const uint8_t f = (sf[m] & 3) | (dirty[l] ? 4 : 0);
    if (f != sf[m])
      fz[c] = f;
    waits = waits || dirty[l];
  }
  const bool any_wrote = __syncthreads_or(wrote);
  const bool any_waits = __syncthreads_or(waits);
  if (threadIdx.x == 0) {
    const int fl = (any_wrote ? 1 : 0) | (any_waits ? 2 : 0);
    tflag[(long)round * ntiles + t] = fl;
    if (fl)
      atomicOr(&flags[round], 1);
  }
}

// ---------------------------------------------------------------------------
// 2D re-distancing as one persistent grid: global Jacobi sweeps of the same
// update (fmm_update), one grid barrier per sweep.  The tiled rounds above
// exchange halos only between launches, so information crosses a tile per
// round and each tile re-sweeps its points until its halo settles (33-91
// updates per cell on the 800 x 400 bubble).  Here every sweep sees the
// previous sweep's values everywhere: a sweep updates only the points whose
// neighbours changed in the previous sweep (a work list), the front moves a
// cell per sweep, and the number of sweeps is the depth of the marcher's
// dependency chain (~1.4 x the largest distance in cells).  Each sweep is
// one FP64 update per listed point (one lane each) and one barrier, so a
// sweep costs about one update's FP64 chain (on GB300 a warp's FP64
// instruction holds its partition's FP64 unit ~64 cycles) plus the barrier.
//
// Jacobi with two buffers: sweep s reads d[s % 2] / par[s % 2] and writes
// d[(s + 1) % 2] / par[(s + 1) % 2] for its listed points; a point that
// changes lists itself for the next sweep as well as its unfrozen
// neighbours, which copies its new value into the other buffer, so after
// sweep s the written buffer holds every point's latest value.  The fixed
// point, and so the result, is that of the tiled form: the sweeps end when
// no point changes, whatever the order of the work.  From sweep mono_from
// on only smaller |d| is taken (termination, as the tiled form's last
// rounds); a list still non-empty after max_sweeps sets err bit 0.
//
// The blocks wait for one another at the barrier, so the kernel is launched
// cooperatively (all blocks resident); each wait is bounded (~1 s), after
// which the block sets err bit 2 and leaves.
struct FmmGlobal {
  double *d[2];
  uint8_t *par[2];
  const uint8_t *fz;
  int *list[2];
  int *qst;           // the sweep a point is listed for (dedupes the lists)
  int *cnt;           // cnt[3]: list lengths, rotating
  unsigned *bar;      // bar + 2: the barrier's two 64-bit words
  int *err;
  int *sweeps;        // optional: receives the sweeps taken
  int mono_from, max_sweeps;
};

// GPU-scope acquire / release accesses (PTX memory model, sm_70 and later).
GPR_D unsigned long long fmm_add_acq_rel64(unsigned long long *p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;"
               : "=l"(old)
               : "l"(p), "l"(v)
               : "memory");
  return old;
}
GPR_D unsigned long long fmm_ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier at the end of sweep s, which also sums the sweep's list
// appends: the 64-bit word words[s % 2] counts the blocks' arrivals (bits
// 40..63) and the entries they appended (bits 0..39) over the sweeps of that
// parity.  Each block arrives once (one thread, an acquire-release add of
// 2^40 + its appends, after the block barrier, which orders the block's
// writes before it) and waits with acquire loads until all blocks have
// arrived for this sweep: nblocks (s / 2 + 1) arrivals.  Two words, so that
// a block already at the next sweep's barrier cannot be counted here.  The
// next list's length is the sum's growth since the previous sweep of the
// same parity (prev[2], kept by the block).  The wait gives up after ~1 s
// (err bit 2).  Returns the length, or -1 after a timeout.
GPR_D int fmm_grid_sync(unsigned long long *words, unsigned nblocks, int s, int appended,
                        unsigned long long prev[2], int *err) {
  __shared__ int shn;
  constexpr unsigned long long ARR = 1ull << 40, CNT = ARR - 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int k = s & 1;
    unsigned long long *w = words + k;
    const unsigned long long target = (unsigned long long)nblocks * (unsigned)(s / 2 + 1);
    unsigned long long v = fmm_add_acq_rel64(w, ARR + (unsigned)appended) + ARR + (unsigned)appended;
    const long long t0 = clock64();
    shn = 0;
    while ((v >> 40) < target) {
      if (clock64() - t0 > 2000000000LL) {  // ~1 s at 2 GHz
        atomicOr(err, 4);
        shn = -1;
        break;
      }
      v = fmm_ld_acquire(w);
    }
    if (shn == 0) {
      shn = (int)((v & CNT) - prev[k]);
      prev[k] = v & CNT;
    }
  }
  __syncthreads();
  return shn;
}

// Lists the candidates cand[k] with want[k] for sweep s, each point once per
// sweep (stamps in qst): the stamps' atomics are issued back to back, and a
// warp reserves its list entries with one atomic.
template <int K>
GPR_D void fmm_enqueue(const bool (&want)[K], const int (&cand)[K], int s, const FmmGlobal &G,
                       int *appended = nullptr) {
  bool mine[K];
#pragma unroll
  for (int k = 0; k < K; k++)
    mine[k] = want[k] ? atomicMax(G.qst + cand[k], s) < s : false;
  int nk = 0;
#pragma unroll
  for (int k = 0; k < K; k++)
    nk += mine[k];
  const int lane = threadIdx.x & 31;
  int incl = nk;  // inclusive warp scan
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o)
      incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0)
    return;
  int base = 0;
  if (lane == 31) {
    base = atomicAdd(G.cnt + s % 3, total);
    if (appended)
      atomicAdd(appended, total);  // the block's appends (shared memory)
  }
  base = __shfl_sync(0xffffffffu, base, 31);
  int pos = base + incl - nk;
  int *lst = G.list[s & 1];
#pragma unroll
  for (int k = 0; k < K; k++)
    if (mine[k])
      lst[pos++] = cand[k];
}

// The first list: unfrozen points next to the frozen band.
__global__ void k_fmm_seed(Grid g, FmmGlobal G, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  bool want[1] = {false};
  if (c < g.ncell && !(G.fz[c] & 1)) {
    const int i = c / g.ny, j = c % g.ny;
    want[0] = (i > 0 && (G.fz[c - g.ny] & 1)) || (i < g.nx - 1 && (G.fz[c + g.ny] & 1)) ||
              (j > 0 && (G.fz[c - 1] & 1)) || (j < g.ny - 1 && (G.fz[c + 1] & 1));
  }
  const int cand[1] = {(int)(c < g.ncell ? c : 0)};
  fmm_enqueue<1>(want, cand, 0, G);
}

__global__ void __launch_bounds__(256) k_fmm_global(Grid g, FmmConst K, FmmGlobal G,
                                                     const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  const unsigned nb = gridDim.x;
  const long nthr = (long)gridDim.x * blockDim.x;
  const long gid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  __shared__ int appended;
  if (threadIdx.x == 0)
    appended = 0;
  unsigned long long prev[2] = {0ull, 0ull};  // used by thread 0
  int s = 0;
  int n = __ldcg(G.cnt);  // the first list (k_fmm_seed)
  for (; s < G.max_sweeps; s++) {
    if (n <= 0)
      break;
    if (gid == 0)
      G.cnt[(s + 2) % 3] = 0;  // the list count of sweep s - 1, no longer read
    const double *src = G.d[s & 1];
    double *dst = G.d[(s + 1) & 1];
    const uint8_t *psrc = G.par[s & 1];
    uint8_t *pdst = G.par[(s + 1) & 1];
    const int *lst = G.list[s & 1];
    const bool mono = s >= G.mono_from;
    // whole warps take list entries, so that the enqueues can aggregate
    const long nround = (n + 31) / 32 * 32;
    for (long q = gid; q < nround; q += nthr) {
      const bool live = q < n;
      const int c = live ? __ldcg(lst + q) : 0;
      const int i = c / g.ny, j = c % g.ny;
      bool chg = false;
      if (live) {
        double nb4[2][2];
        bool bd[2][2], ex[2][2];
        const long cn[2][2] = {{c - g.ny, c + g.ny}, {c - 1, c + 1}};
        const bool in[2][2] = {{i > 0, i < g.nx - 1}, {j > 0, j < g.ny - 1}};
        // a neighbour that recorded this point as entered (its bit for the
        // opposite side) is not a candidate: bits 2 dim + side
        const int xb[2][2] = {{1, 0}, {3, 2}};
        for (int dim = 0; dim < 2; dim++)
          for (int sd = 0; sd < 2; sd++) {
            const bool ok = in[dim][sd];
            const long m = ok ? cn[dim][sd] : c;
            nb4[dim][sd] = ok ? __ldcg(src + m) : INFINITY;
            bd[dim][sd] = ok && (G.fz[m] & 1);
            ex[dim][sd] = ok && ((__ldcg(psrc + m) >> xb[dim][sd]) & 1);
          }
        const double old = __ldcg(src + c);
        const uint8_t pold = __ldcg(psrc + c);
        int msk;
        const double nv = fmm_update(nb4, bd, ex, (G.fz[c] & 2) != 0, 2, old, K, msk);
        chg = mono ? fabs(nv) < fabs(old) : (nv != old || (uint8_t)msk != pold);
        __stcg(dst + c, chg ? nv : old);
        __stcg(pdst + c, chg ? (uint8_t)msk : pold);
      }
      // list the point itself and its unfrozen neighbours for sweep s + 1
      const int cand[5] = {c, i > 0 ? c - g.ny : c, i < g.nx - 1 ? c + g.ny : c,
                           j > 0 ? c - 1 : c, j < g.ny - 1 ? c + 1 : c};
      bool want[5] = {chg, chg && i > 0, chg && i < g.nx - 1, chg && j > 0, chg && j < g.ny - 1};
#pragma unroll
      for (int k = 1; k < 5; k++)
        want[k] = want[k] && !(G.fz[cand[k]] & 1);
      fmm_enqueue<5>(want, cand, s + 1, G, &appended);
    }
    __syncthreads();
    const int app = appended;
    __syncthreads();
    if (threadIdx.x == 0)
      appended = 0;
    n = fmm_grid_sync((unsigned long long *)(G.bar + 2), nb, s, app, prev, G.err);
    if (n < 0)
      return;
  }
  if (gid == 0 && s >= G.max_sweeps && n != 0)
    atomicOr(G.err, 1);  // not converged within the sweep budget
  if (gid == 0) {
    G.cnt[3] = s;  // the sweeps taken
    if (G.sweeps)
      *G.sweeps = s;
  }
}

// Final values (base_marcher.cpp:103-106, 190-196): zeros when nothing
// froze, DBL_MAX where the march never arrived; the distance also replaces
// the level set in u (renormalize_levelsets, multi/functions.cpp:56-64).
template <int V>
__global__ void k_fmm_finish(double *__restrict__ d, double *__restrict__ u, long ncell,
                             const int *__restrict__ anyfrozen, const int *__restrict__ flags,
                             int last, int *__restrict__ err, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c == 0 && flags[last] != 0)
    atomicOr(err, 1);  // not converged within the round budget
  if (c >= ncell)
    return;
  double x = d[c];
  if (isinf(x))
    x = DBL_MAX;
  if (!*anyfrozen)
    x = 0.0;
  d[c] = x;
  if (u)
    u[c * V + V - 1] = x;
}

// ===========================================================================
// Normals and interface cells of one material from its level set phi
// (material_indicator, multi/functions.cpp:66-81: phi = +-u's level set for
// two materials; the material occupies phi <= 0).

__global__ void k_mat_phi(const double *__restrict__ d, int sgn, double *__restrict__ phim,
                          long ncell, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c < ncell)
    phim[c] = sgn > 0 ? d[c] : -d[c];
}

// finite_difference (multi/functions.cpp:16-54): central differences, the
// first and last rows (columns) copied from their neighbours.  dphi is
// [ncell][nd].
__global__ void k_finite_difference(const double *__restrict__ phi, double *__restrict__ dphi,
                                    Grid g, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= g.ncell)
    return;
  if (g.nd == 1) {
    int i = (int)c, ii = i == 0 ? 1 : (i == g.nx - 1 ? g.nx - 2 : i);
    dphi[c] = dvd(sub(phi[ii + 1], phi[ii - 1]), mul(2.0, g.dx));
    return;
  }
  int i = (int)(c / g.ny), j = (int)(c % g.ny);
  int ii = i == 0 ? 1 : (i == g.nx - 1 ? g.nx - 2 : i);
  int jj = j == 0 ? 1 : (j == g.ny - 1 ? g.ny - 2 : j);
  dphi[2 * c] = dvd(sub(phi[(long)(ii + 1) * g.ny + j], phi[(long)(ii - 1) * g.ny + j]),
                    mul(2.0, g.dx));
  dphi[2 * c + 1] = dvd(sub(phi[(long)i * g.ny + jj + 1], phi[(long)i * g.ny + jj - 1]),
                        mul(2.0, g.dy));
}

// find_interface_cells (multi/fill.cpp:20-74), gathered per cell: the
// reference's scatter only ever writes sign(phi) of the written cell, or -2
// for an isolated phi <= 0 cell, so each cell's final value follows from its
// own neighbourhood.
GPR_D bool nonisolated(const double *phi, int i, int j, const Grid &g) {
  long c = (long)i * g.ny + j;
  return (i > 0 && phi[c - g.ny] <= 0.0) || (i < g.nx - 1 && phi[c + g.ny] <= 0.0) ||
         (j > 0 && phi[c - 1] <= 0.0) || (j < g.ny - 1 && phi[c + 1] <= 0.0);
}

__global__ void k_interface_cells(const double *__restrict__ phi, int32_t *__restrict__ im,
                                  Grid g, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= g.ncell)
    return;
  double p = phi[c];
  int sg = p <= 0.0 ? -1 : 1;
  if (g.nd == 1) {
    int i = (int)c;
    bool hit = (i > 0 && mul(phi[c - 1], p) <= 0.0) ||
               (i < g.nx - 1 && mul(p, phi[c + 1]) <= 0.0);
    im[c] = hit ? sg : 0;
    return;
  }
  int i = (int)(c / g.ny), j = (int)(c % g.ny);
  long nbr[4] = {i > 0 ? c - g.ny : -1, i < g.nx - 1 ? c + g.ny : -1, j > 0 ? c - 1 : -1,
                 j < g.ny - 1 ? c + 1 : -1};
  int ni[4] = {i - 1, i + 1, i, i}, nj[4] = {j, j, j - 1, j + 1};
  int out = 0;
  if (p <= 0.0) {
    if (!nonisolated(phi, i, j, g)) {
      im[c] = -2;
      return;
    }
    for (int q = 0; q < 4; q++)
      if (nbr[q] >= 0 && mul(p, phi[nbr[q]]) <= 0.0)
        out = -1;
  }
  // written by a non-isolated phi <= 0 neighbour whose product with us is <= 0
  for (int q = 0; q < 4 && out == 0; q++) {
    if (nbr[q] < 0)
      continue;
    double pn = phi[nbr[q]];
    if (pn <= 0.0 && mul(pn, p) <= 0.0 && nonisolated(phi, ni[q], nj[q], g))
      out = sg;
  }
  im[c] = out;
}

// ===========================================================================
// Interface Riemann problem (slip conditions, no heat conduction).

// rotation_matrix (rotations.cpp:5-35): rows e1 = n, e2, e3.
GPR_D void rotation(const double n[2], int nd, double R[3][3]) {
  double e1[3] = {n[0], nd == 2 ? n[1] : 0.0, 0.0}, e2[3], e3[3], den;
  double Sq = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  if (fabs(e1[1] + e1[2]) <= fabs(e1[1] - e1[2])) {
    den = sqrt(2.0 * (1.0 - e1[0] * e1[1] - e1[1] * e1[2] - e1[2] * e1[0]));
    e2[0] = e1[1] - e1[2];
    e2[1] = e1[2] - e1[0];
    e2[2] = e1[0] - e1[1];
    double Sum = e1[0] + e1[1] + e1[2];
    for (int i = 0; i < 3; i++)
      e3[i] = e1[i] * Sum - Sq;
  } else {
    den = sqrt(2.0 * (1.0 + e1[0] * e1[1] + e1[1] * e1[2] - e1[2] * e1[0]));
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

// rotate_tensors (rotations.cpp:37-47): v <- R v, A <- R A R^T.
GPR_D void rotate(double *Q, const double R[3][3]) {
  double v[3], T[9];
  for (int i = 0; i < 3; i++)
    v[i] = R[i][0] * Q[2] + R[i][1] * Q[3] + R[i][2] * Q[4];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      T[3 * i + j] = R[i][0] * Q[5 + j] + R[i][1] * Q[8 + j] + R[i][2] * Q[11 + j];
  for (int i = 0; i < 3; i++) {
    Q[2 + i] = v[i];
    for (int j = 0; j < 3; j++)
      Q[5 + 3 * i + j] = T[3 * i] * R[j][0] + T[3 * i + 1] * R[j][1] + T[3 * i + 2] * R[j][2];
  }
}

// Gaussian elimination with partial pivoting: A X = B in place (A n x n,
// B n x m, row-major).  Returns false on a zero pivot.
template <int n, int m> GPR_D bool gauss(double *A, double *B) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (fabs(A[r * n + c]) > fabs(A[p * n + c]))
        p = r;
    if (A[p * n + c] == 0.0)
      return false;
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
  return true;
}

GPR_D bool inv3(const double *M, double *out) {
  double A[9];
  for (int k = 0; k < 9; k++) {
    A[k] = M[k];
    out[k] = (k % 4) == 0 ? 1.0 : 0.0;
  }
  return gauss<3, 3>(A, out);
}

// Eigenvalues of a real 3 x 3 matrix from its characteristic polynomial
// (depressed cubic: trigonometric form for three real roots, Cardano for a
// complex pair).  ok = false when an eigenvalue has a non-positive real part
// or the pair's imaginary part exceeds 1e-6 of the spectral radius: the
// reference's Q diag(Re(lambda)^(-1/2)) Q^(-1) with Q = Re(eigenvectors)
// (riemann.cpp:136-141) is NaN or singular there and its star state falls
// back to the input state.
GPR_D bool eig3_real_positive(const double *M) {
  double p1 = M[0] + M[4] + M[8];
  double p2 = M[0] * M[4] - M[1] * M[3] + M[0] * M[8] - M[2] * M[6] + M[4] * M[8] -
              M[5] * M[7];
  double p3 = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
              M[2] * (M[3] * M[7] - M[4] * M[6]);
  double s = p1 / 3.0;
  double a = p2 - p1 * p1 / 3.0;
  double b = -2.0 * p1 * p1 * p1 / 27.0 + p1 * p2 / 3.0 - p3;
  double disc = b * b / 4.0 + a * a * a / 27.0;  // > 0: complex pair
  if (disc > 0.0) {
    double sq = sqrt(disc);
    double u = cbrt(-b / 2.0 + sq), v = cbrt(-b / 2.0 - sq);
    double lr = s + u + v;                  // real root
    double cr = s - (u + v) / 2.0;          // real part of the pair
    double ci = 0.86602540378443864676 * fabs(u - v);
    double rad = fmax(fabs(lr), hypot(cr, ci));
    return lr > 0.0 && cr > 0.0 && !(ci > 1e-6 * rad);
  }
  // three real roots: s + 2 sqrt(-a/3) cos(theta/3 - 2 pi k / 3)
  double r = sqrt(fmax(-a / 3.0, 0.0));
  double lo;
  if (r == 0.0) {
    lo = s;
  } else {
    double ct = -b / (2.0 * r * r * r);
    ct = fmin(1.0, fmax(-1.0, ct));
    double th = acos(ct);
    // the smallest of the three is k = 1 (theta / 3 + 2 pi / 3 in [2pi/3, pi])
    lo = s + 2.0 * r * cos(th / 3.0 + 2.0943951023931954923);
  }
  return lo > 0.0;
}

// Inverse principal square root by the Denman-Beavers iteration
// (Y -> M^(1/2), Z -> M^(-1/2)); the reference forms the same matrix
// function from an eigen-decomposition (riemann.cpp:136-141).
GPR_D bool inv_sqrt3(const double *M, double *Zout) {
  double Y[9], Z[9], Yi[9], Zi[9];
  for (int k = 0; k < 9; k++) {
    Y[k] = M[k];
    Z[k] = (k % 4) == 0 ? 1.0 : 0.0;
  }
  int extra = 0;
  for (int it = 0; it < 100; it++) {
    if (!inv3(Y, Yi) || !inv3(Z, Zi))
      return false;
    double dmax = 0.0, ymax = 0.0;
    for (int k = 0; k < 9; k++) {
      double y = 0.5 * (Y[k] + Zi[k]);
      double z = 0.5 * (Z[k] + Yi[k]);
      dmax = fmax(dmax, fabs(y - Y[k]));
      ymax = fmax(ymax, fabs(y));
      Y[k] = y;
      Z[k] = z;
    }
    if (dmax <= 1e-13 * ymax && ++extra == 2)
      break;
  }
  for (int k = 0; k < 9; k++)
    Zout[k] = Z[k];
  return true;
}

// Total stress column 0: Sigma = p e0 - sigma(:, 0)  (variables/state.cpp:39-46).
GPR_D void Sigma0(const double *Q, const Prim<false> &s, double *S) {
  sigma_col<false>(Q, s, 0, S);
  S[0] = s.p - S[0];
  S[1] = -S[1];
  S[2] = -S[2];
}

// d sigma(:, 0) / d rho and d sigma(:, 0) / dA (variables/state.cpp:43-56,
// energy/derivatives.cpp).
GPR_D void dsigma0(const double *Q, const Prim<false> &s, const DevPar &P, double *sr,
                   double *Pi1) {
  double r = s.r;
  double dcs2 = P.beta / r * s.cs2;
  sigma_col<false>(Q, s, 0, sr);
  double f = 1.0 / r + dcs2 / s.cs2;
  for (int i = 0; i < 3; i++)
    sr[i] *= f;
  const double *A = Q + 5;
  double G[9], ret[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      G[3 * i + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  for (int k = 0; k < 9; k++)
    ret[k] = s.AdG[k];
  for (int i = 0; i < 3; i++)
    ret[3 * i] *= 2.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      ret[3 * i + j] += 1.0 / 3.0 * A[3 * i] * G[j];
  for (int k = 0; k < 9; k++)
    ret[k] += G[0] * A[k];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      Pi1[3 * i + j] = -r * s.cs2 * ret[3 * j + i];
}

// c_0 (waves/speeds.cpp:8-18).
GPR_D double c0_of(const Prim<false> &s, const DevPar &P) {
  double r = s.r, G = s.e.G, dG = s.e.dG;
  double dedrho = s.e.der - (s.e.dpr * r * G + (G + r * dG) * (s.p - s.e.pr)) /
                                ((r * G) * (r * G));
  double dcs2 = P.beta / r * s.cs2;
  double dC0 = (1.0 - P.beta / G) * dcs2 + P.beta / (G * G) * dG * s.cs2;
  double dEdr = dedrho + dC0 / 4.0 * s.devGsq;
  double dedp = 1.0 / (r * G);
  return sqrt((s.p / (r * r) - dEdr) / dedp);
}

// The first three columns of riemann_constraints (riemann.cpp:79-154) for
// the non-thermal system; rows 0-4 are X, rows 11-13 -sgn Y0 Xi1 X, the rest
// zero (the other columns multiply zero coefficients in star_stepper).
// Rx is [5][3], Ry is [3][3].
GPR_D bool constraints(const double *Q, double sgn, const DevPar &P, double *Rx, double *Ry) {
  Prim<false> s;
  prim<false>(Q, P, s);
  double r = s.r;
  const double *A = Q + 5;
  double sr[3], Pi1[9], Pi1i[9], Ai[9], sg[3];
  dsigma0(Q, s, P, sr, Pi1);
  sigma_col<false>(Q, s, 0, sg);
  if (!inv3(A, Ai) || !inv3(Pi1, Pi1i))
    return false;
  double tmp[25];
  for (int k = 0; k < 25; k++)
    tmp[k] = 0.0;
  for (int i = 0; i < 3; i++) {
    tmp[5 * i] = -sr[i];
    for (int j = 0; j < 3; j++)
      tmp[5 * i + 2 + j] = -Pi1[3 * i + j];
  }
  tmp[1] = 1.0;
  double c0 = c0_of(s, P);
  double B[6] = {r, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int j = 0; j < 3; j++)
    B[3 + j] = sg[j] - r * sr[j];
  B[3] += r * c0 * c0;
  double C[6];
  for (int i = 0; i < 3; i++) {
    C[2 * i] = -(Pi1i[3 * i] * sr[0] + Pi1i[3 * i + 1] * sr[1] + Pi1i[3 * i + 2] * sr[2]);
    C[2 * i + 1] = Pi1i[3 * i];
  }
  double BA[6];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 3; j++)
      BA[3 * i + j] = B[3 * i] * Ai[j] + B[3 * i + 1] * Ai[3 + j] + B[3 * i + 2] * Ai[6 + j];
  double Z[4];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      Z[2 * i + j] = (i == j ? 1.0 : 0.0) -
                     (BA[3 * i] * C[j] + BA[3 * i + 1] * C[2 + j] + BA[3 * i + 2] * C[4 + j]);
  double dz = Z[0] * Z[3] - Z[1] * Z[2];
  if (dz == 0.0)
    return false;
  double Zi[4] = {Z[3] / dz, -Z[1] / dz, -Z[2] / dz, Z[0] / dz};
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 5; j++) {
      double w0 = j == 0 ? 1.0 : (j == 1 ? 0.0 : -BA[j - 2]);
      double w1 = j == 0 ? 0.0 : (j == 1 ? 1.0 : -BA[3 + j - 2]);
      tmp[5 * (3 + i) + j] = Zi[2 * i] * w0 + Zi[2 * i + 1] * w1;
    }
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 3; j++)
      Rx[3 * i + j] = i == j ? 1.0 : 0.0;
  if (!gauss<5, 3>(tmp, Rx))
    return false;
  // Xi1 (3 x 5) and Xi2 (5 x 3) of system/eig.cpp:8-53 along x
  double X1[15], X2[15], Xi[9], Y0[9];
  for (int k = 0; k < 15; k++)
    X1[k] = X2[k] = 0.0;
  X1[1] = 1.0 / r;
  for (int i = 0; i < 3; i++) {
    X1[5 * i] = -1.0 / r * sr[i];
    for (int j = 0; j < 3; j++)
      X1[5 * i + 2 + j] = -1.0 / r * Pi1[3 * i + j];
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
      double t = 0.0;
      for (int k = 0; k < 5; k++)
        t += X1[5 * i + k] * X2[3 * k + j];
      Xi[3 * i + j] = t;
    }
  if (!eig3_real_positive(Xi) || !inv_sqrt3(Xi, Y0))
    return false;
  double X1X[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double t = 0.0;
      for (int k = 0; k < 5; k++)
        t += X1[5 * i + k] * Rx[3 * k + j];
      X1X[3 * i + j] = t;
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      Ry[3 * i + j] = -sgn * (Y0[3 * i] * X1X[j] + Y0[3 * i + 1] * X1X[3 + j] +
                              Y0[3 * i + 2] * X1X[6 + j]);
  return true;
}

// Cvec_to_Pvec + P += R c + Pvec_to_Cvec (functions/vectors.cpp:85-154,
// riemann.cpp:191-200) for the non-thermal layout
// P = [rho, p, A(:,0), A(:,1), A(:,2), v, phi].
GPR_D void apply_correction(double *Q, const double *Rx, const double *Ry, const double *cc,
                            const DevPar &P) {
  Prim<false> s;
  prim<false>(Q, P, s);
  double Pv[14];
  Pv[0] = Q[0];
  Pv[1] = s.p;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      Pv[2 + 3 * j + i] = Q[5 + 3 * i + j];
  for (int i = 0; i < 3; i++)
    Pv[11 + i] = Q[2 + i] * s.ir;
  for (int k = 0; k < 5; k++)
    Pv[k] += Rx[3 * k] * cc[0] + Rx[3 * k + 1] * cc[1] + Rx[3 * k + 2] * cc[2];
  for (int k = 0; k < 3; k++)
    Pv[11 + k] += Ry[3 * k] * cc[0] + Ry[3 * k + 1] * cc[1] + Ry[3 * k + 2] * cc[2];
  double r = Pv[0], p = Pv[1];
  Q[0] = r;
  double A[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      A[3 * i + j] = Pv[2 + 3 * j + i];
  for (int k = 0; k < 9; k++)
    Q[5 + k] = A[k];
  double v0 = Pv[11], v1 = Pv[12], v2 = Pv[13];
  Q[2] = r * v0;
  Q[3] = r * v1;
  Q[4] = r * v2;
  // total_energy (energy/eos.cpp:43-47)
  double ir = 1.0 / r;
  EosRho e = eos_rho(r, ir, P);
  double cs2 = P.beta == 0.0 ? P.b02 : P.b02 * pow(r * P.ir0, P.beta);
  double C0 = (1.0 - P.beta / e.G) * cs2;
  double G00 = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  double G11 = A[3] * A[3] + A[4] * A[4] + A[5] * A[5];
  double G22 = A[6] * A[6] + A[7] * A[7] + A[8] * A[8];
  double G01 = A[0] * A[3] + A[1] * A[4] + A[2] * A[5];
  double G02 = A[0] * A[6] + A[1] * A[7] + A[2] * A[8];
  double G12 = A[3] * A[6] + A[4] * A[7] + A[5] * A[8];
  double t = (G00 + G11 + G22) / 3.0;
  double dg = (G00 - t) * (G00 - t) + (G11 - t) * (G11 - t) + (G22 - t) * (G22 - t) +
              2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
  double E = e.er + (p - e.pr) / (r * e.G) + 0.5 * (v0 * v0 + v1 * v1 + v2 * v2) +
             C0 / 4.0 * dg;
  Q[1] = r * E;
}

constexpr double STAR_TOL = 1e-8;  // options.h:22

// check_star_convergence (riemann.cpp:26-77), slip conditions.
GPR_D bool star_converged(const double *QL, const double *QR, const DevPar &PL,
                          const DevPar &PR) {
  Prim<false> sl;
  prim<false>(QL, PL, sl);
  double SL[3];
  Sigma0(QL, sl, SL);
  if (PR.EOS > -1) {
    Prim<false> sr;
    prim<false>(QR, PR, sr);
    double SR[3];
    Sigma0(QR, sr, SR);
    double r0 = fmin(PL.rho0, PR.rho0), b02 = fmin(PL.b02, PR.b02);
    return fabs(SL[0] - SR[0]) / (b02 * r0) < STAR_TOL &&
           fabs(QL[2] / QL[0] - QR[2] / QR[0]) / sqrt(b02) < STAR_TOL;
  }
  double mx = fmax(fabs(SL[0]), fmax(fabs(SL[1]), fabs(SL[2])));
  return mx / (PL.b02 * PL.rho0) < STAR_TOL;
}

// star_stepper (riemann.cpp:156-201) with slip_bcs (conditions.cpp:31-64).
GPR_D bool star_step(double *QL, double *QR, const DevPar &PL, const DevPar &PR) {
  double RLx[15], RLy[9], cL[3];
  if (!constraints(QL, 1.0, PL, RLx, RLy))
    return false;
  Prim<false> sl;
  prim<false>(QL, PL, sl);
  double xL[3];
  Sigma0(QL, sl, xL);
  if (PR.EOS > -1) {
    double RRx[15], RRy[9], xR[3], cR[3];
    if (!constraints(QR, -1.0, PR, RRx, RRy))
      return false;
    Prim<false> sr;
    prim<false>(QR, PR, sr);
    Sigma0(QR, sr, xR);
    double yL = QL[2] / QL[0], yR = QR[2] / QR[0];
    // row 11 of the constraint matrices (the normal velocity)
    double dL = RLy[0] * xL[0] + RLy[1] * xL[1] + RLy[2] * xL[2];
    double dR = RRy[0] * xR[0] + RRy[1] * xR[1] + RRy[2] * xR[2];
    double x0 = (yR - yL + dL - dR) / (RLy[0] - RRy[0]);
    double xs[3] = {x0, 0.0, 0.0};
    for (int i = 0; i < 3; i++) {
      cL[i] = xs[i] - xL[i];
      cR[i] = xs[i] - xR[i];
    }
    apply_correction(QR, RRx, RRy, cR, PR);
  } else {
    for (int i = 0; i < 3; i++)
      cL[i] = -xL[i];
    for (int k = 0; k < 14; k++)
      QR[k] = 0.0;
  }
  apply_correction(QL, RLx, RLy, cL, PL);
  return true;
}

// left_star_state (riemann.cpp:203-233): the left star state of the
// interface Riemann problem between QL (material PL) and QR (material PR)
// along the unit normal n: at most ten linearised steps, each after a half
// step dt/2 of the stiff relaxation; the input is returned if a NaN appears.
// The level set entry (index 14) is carried through unchanged.
GPR_D void left_star_state(const double *QL0, const double *QR0, const DevPar &PL,
                           const DevPar &PR, double dt, const double n[2], int nd,
                           double *out) {
  double QL[15], QR[15], R[3][3];
  for (int k = 0; k < 15; k++) {
    QL[k] = QL0[k];
    QR[k] = QR0[k];
  }
  rotation(n, nd, R);
  rotate(QL, R);
  rotate(QR, R);
  bool nan = false;
  for (int count = 0; count < 10 && !star_converged(QL, QR, PL, PR); count++) {
    // ode_stepper_analytic (relaxation/analytic.cpp:152-161), no heat flux
    QL[2] += PL.dp0 * dt / 2;
    QL[3] += PL.dp1 * dt / 2;
    QL[4] += PL.dp2 * dt / 2;
    ode_distortion(QL, dt / 2, PL);
    if (PR.EOS > -1) {
      QR[2] += PR.dp0 * dt / 2;
      QR[3] += PR.dp1 * dt / 2;
      QR[4] += PR.dp2 * dt / 2;
      ode_distortion(QR, dt / 2, PR);
    }
    if (!star_step(QL, QR, PL, PR)) {
      nan = true;
      break;
    }
  }
  for (int k = 0; k < 15; k++)
    nan = nan || isnan(QL[k]);
  if (nan) {
    for (int k = 0; k < 15; k++)
      out[k] = QL0[k];
    return;
  }
  double RT[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      RT[i][j] = R[j][i];
  rotate(QL, RT);
  for (int k = 0; k < 15; k++)
    out[k] = QL[k];
}

// ===========================================================================
// Boundary fill (multi/fill.cpp:96-235).

// One boundary cell (intMask == 1: the first ghost cell outside material
// mat) and where its fill reads and writes.
struct BPlan {
  int c;       // the cell
  int R;       // probe on the far side of the interface (QR)
  int ql;      // cell QL is read from
  int wi;      // interface cell also written (-1: none)
  int miR;     // material of QR
  int pad;
  double n[2]; // normal (axis-aligned by the fallback branch)
};

// get_material_index (functions/vectors.cpp:24-31) from the level set entry.
template <int V> GPR_D int mat_of(const double *grid, long c) {
  return grid[c * V + V - 1] >= 0.0 ? 1 : 0;
}

// Unit normal of dphi row c (normal, multi/functions.cpp:14); false when it
// is not finite.
GPR_D bool unit_normal(const double *dphi, long c, int nd, double n[2]) {
  if (nd == 1) {
    double g = dphi[c];
    double s = __dsqrt_rn(mul(g, g));
    n[0] = dvd(g, s);
    n[1] = 0.0;
    return isfinite(n[0]);
  }
  double g0 = dphi[2 * c], g1 = dphi[2 * c + 1];
  double s = __dsqrt_rn(add(mul(g0, g0), mul(g1, g1)));
  n[0] = dvd(g0, s);
  n[1] = dvd(g1, s);
  return isfinite(n[0]) && isfinite(n[1]);
}

// Plans every boundary cell: boundary_inds (fill.cpp:96-132) and the choice
// of QL in fill_boundary_inner (fill.cpp:134-198).  Cells whose fill would
// read outside the grid in the reference are counted in err[1] and left
// unfilled.  lastw[x] collects the largest boundary cell writing x.
template <int V>
__global__ void k_plan(const double *__restrict__ phi, const double *__restrict__ dphi,
                       const int32_t *__restrict__ im, const double *__restrict__ grid,
                       int mat, Grid g,
                       BPlan *__restrict__ plan, int *__restrict__ nplan,
                       int32_t *__restrict__ pidx, int32_t *__restrict__ lastw,
                       int *__restrict__ err, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= g.ncell || im[c] != 1)
    return;
  int i = g.nd == 1 ? (int)c : (int)(c / g.ny), j = g.nd == 1 ? 0 : (int)(c % g.ny);
  double n[2];
  if (!unit_normal(dphi, c, g.nd, n)) {
    atomicAdd(&err[1], 1);
    return;
  }
  double phii = phi[c];
  int vi[2], vl[2], vr[2];
  int ind2[2] = {i, j};
  for (int k = 0; k < g.nd; k++) {
    double h = k == 0 ? g.dx : g.dy;
    double xp = mul(add((double)ind2[k], 0.5), h);
    double xi = sub(xp, mul(phii, n[k]));
    double hn = mul(mul(1.0, h), n[k]);
    vi[k] = (int)dvd(xi, h);
    vl[k] = (int)dvd(sub(xi, hn), h);
    vr[k] = (int)dvd(add(xi, hn), h);
  }
  long interf = g.nd == 1 ? vi[0] : (long)vi[0] * g.ny + vi[1];
  long L = g.nd == 1 ? vl[0] : (long)vl[0] * g.ny + vl[1];
  long R = g.nd == 1 ? vr[0] : (long)vr[0] * g.ny + vr[1];
  if (interf < 0 || interf >= g.ncell || L < 0 || L >= g.ncell || R < 0 || R >= g.ncell) {
    atomicAdd(&err[1], 1);
    return;
  }
  long ql;
  if (mat_of<V>(grid, interf) == mat) {
    ql = interf;
  } else if (mat_of<V>(grid, L) == mat) {
    ql = L;
  } else {
    if (g.nd == 1) {
      atomicAdd(&err[1], 1);
      return;
    }
    int Li[2] = {i, j};
    long Lind;
    int n0 = (n[0] > 0) - (n[0] < 0), n1 = (n[1] > 0) - (n[1] < 0);
    if (fabs(n[0]) > fabs(n[1])) {
      Li[0] -= n0;
      Lind = (long)Li[0] * g.ny + Li[1];
      if (Lind >= 0 && Lind < g.ncell && mat_of<V>(grid, Lind) == mat) {
        n[0] = n0;
        n[1] = 0.0;
      } else {
        Li[0] += n0;
        Li[1] -= n1;
        Lind = (long)Li[0] * g.ny + Li[1];
        n[0] = 0.0;
        n[1] = n1;
      }
    } else {
      Li[1] -= n1;
      Lind = (long)Li[0] * g.ny + Li[1];
      if (Lind >= 0 && Lind < g.ncell && mat_of<V>(grid, Lind) == mat) {
        n[0] = 0.0;
        n[1] = n1;
      } else {
        Li[0] -= n0;
        Li[1] += n1;
        Lind = (long)Li[0] * g.ny + Li[1];
        n[0] = n0;
        n[1] = 0.0;
      }
    }
    if (Lind < 0 || Lind >= g.ncell) {
      atomicAdd(&err[1], 1);
      return;
    }
    if (mat_of<V>(grid, Lind) == mat) {
      ql = Lind;
    } else {
      // neighbor_index(intMask, i, j, nx, ny, -1) (fill.cpp:76-94): the
      // last of left, right, down, up with intMask -1
      long indn = -1;
      if (i > 0 && im[c - g.ny] == -1)
        indn = c - g.ny;
      if (i < g.nx - 1 && im[c + g.ny] == -1)
        indn = c + g.ny;
      if (j > 0 && im[c - 1] == -1)
        indn = c - 1;
      if (j < g.ny - 1 && im[c + 1] == -1)
        indn = c + 1;
      if (indn < 0) {
        atomicAdd(&err[1], 1);
        return;
      }
      ql = indn;
    }
  }
  int k = atomicAdd(nplan, 1);
  BPlan b;
  b.c = (int)c;
  b.R = (int)R;
  b.ql = (int)ql;
  b.wi = mat_of<V>(grid, interf) != mat ? (int)interf : -1;
  b.miR = mat_of<V>(grid, R);
  b.pad = 0;
  b.n[0] = n[0];
  b.n[1] = n[1];
  plan[k] = b;
  pidx[c] = k;
  atomicMax(&lastw[c], (int)c);
  if (b.wi >= 0)
    atomicMax(&lastw[b.wi], (int)c);
}

// For each plan entry, the entry whose fill last wrote its QR cell earlier
// in the reference's (i, j) sweep (-1: QR is the original state), and its
// level in that dependency chain.
__global__ void k_plan_deps(const BPlan *__restrict__ plan, const int *__restrict__ nplan,
                            const int32_t *__restrict__ pidx,
                            const int32_t *__restrict__ lastw, int32_t *__restrict__ dep,
                            const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  int B = *nplan;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < B; k += gridDim.x * blockDim.x) {
    int c = plan[k].c, R = plan[k].R;
    int w = lastw[R];
    int dk = -1;
    if (w >= 0 && w < c) {
      dk = pidx[w];
    } else if (w >= c) {
      // a later (or this) cell writes R too: scan for the last earlier one
      int best = -1;
      for (int q = 0; q < B; q++) {
        int cq = plan[q].c;
        if (cq < c && cq > best && (cq == R || plan[q].wi == R))
          best = cq;
      }
      dk = best >= 0 ? pidx[best] : -1;
    }
    dep[k] = dk;
  }
}

__global__ void k_plan_levels(const int *__restrict__ nplan, const int32_t *__restrict__ dep,
                              int32_t *__restrict__ level, int *__restrict__ maxlevel,
                              const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  int B = *nplan;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < B; k += gridDim.x * blockDim.x) {
    int L = 0, q = dep[k];
    while (q >= 0 && L < B) {
      L++;
      q = dep[q];
    }
    level[k] = L;
    if (L > 0)
      atomicMax(maxlevel, L);
  }
}

template <int V>
GPR_D void solve_plan(int k, const BPlan *plan, const int32_t *dep, const double *grid,
                      double *star, const DevPar &P0, const DevPar &P1, int mat, double dt,
                      int nd) {
  static_assert(V == 15, "the ghost fill is for the viscous one-level-set layout");
  const BPlan &b = plan[k];
  double QL[V], QR[V], out[V];
  for (int v = 0; v < V; v++)
    QL[v] = grid[(long)b.ql * V + v];
  int dk = dep[k];
  for (int v = 0; v < V; v++)
    QR[v] = dk >= 0 && v < V - 1 ? star[(long)dk * V + v] : grid[(long)b.R * V + v];
  const DevPar &PL = mat == 0 ? P0 : P1;
  const DevPar &PR = b.miR == 0 ? P0 : P1;
  left_star_state(QL, QR, PL, PR, dt, b.n, nd, out);
  for (int v = 0; v < V; v++)
    star[(long)k * V + v] = out[v];
}

// Star states of the plan entries on level 0 (all independent).
template <int V>
__global__ void __launch_bounds__(64)
    k_star_level0(const BPlan *__restrict__ plan, const int *__restrict__ nplan,
                  const int32_t *__restrict__ dep, const int32_t *__restrict__ level,
                  const double *__restrict__ grid, double *__restrict__ star, DevPar P0,
                  DevPar P1, int mat, double dt, const double *__restrict__ dt_dev, int nd,
                  const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  if (dt_dev)
    dt = *dt_dev;
  int B = *nplan;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < B; k += gridDim.x * blockDim.x)
    if (level[k] == 0)
      solve_plan<V>(k, plan, dep, grid, star, P0, P1, mat, dt, nd);
}

// Deeper levels, in order, in one block (rare: only where a boundary cell's
// far-side probe was filled earlier in the sweep).
template <int V>
__global__ void __launch_bounds__(64)
    k_star_levels(const BPlan *__restrict__ plan, const int *__restrict__ nplan,
                  const int32_t *__restrict__ dep, const int32_t *__restrict__ level,
                  const int *__restrict__ maxlevel, const double *__restrict__ grid,
                  double *__restrict__ star, DevPar P0, DevPar P1, int mat, double dt,
                  const double *__restrict__ dt_dev, int nd, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  if (dt_dev)
    dt = *dt_dev;
  int B = *nplan, ML = *maxlevel;
  for (int L = 1; L <= ML; L++) {
    for (int k = threadIdx.x; k < B; k += blockDim.x)
      if (level[k] == L)
        solve_plan<V>(k, plan, dep, grid, star, P0, P1, mat, dt, nd);
    __syncthreads();
  }
}

// Every written cell takes the star state of its last writer in the sweep;
// the level set entry keeps the grid's value (fill.cpp:194-197).
template <int V>
__global__ void k_scatter(const BPlan *__restrict__ plan, const int *__restrict__ nplan,
                          const int32_t *__restrict__ lastw, const double *__restrict__ star,
                          double *__restrict__ grid, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  int B = *nplan;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < B; k += gridDim.x * blockDim.x) {
    int c = plan[k].c, wi = plan[k].wi;
    if (lastw[c] == c)
      for (int v = 0; v < V - 1; v++)
        grid[(long)c * V + v] = star[(long)k * V + v];
    if (wi >= 0 && lastw[wi] == c)
      for (int v = 0; v < V - 1; v++)
        grid[(long)wi * V + v] = star[(long)k * V + v];
  }
}

// ===========================================================================
// Layered fill (fill_neighbor_cells, multi/fill.cpp:237-328): layer N0 + 1
// is every cell with intMask 0 (or -2 in 2D) next to a layer-N0 cell.

struct Layer {
  const int32_t *m;  // intMask before this layer
  Grid g;
  int N0;
  GPR_D bool open(long x) const {
    int v = m[x];
    return v == 0 || (g.nd == 2 && v == -2);
  }
  // is x in this layer; indn = the reference's neighbour index (the last
  // match in the order left, right, down, up)
  GPR_D bool in(long x, long &indn) const {
    indn = -1;
    if (!open(x))
      return false;
    if (g.nd == 1) {
      int i = (int)x;
      if (i > 0 && m[x - 1] == N0)
        indn = x - 1;
      if (i < g.nx - 1 && m[x + 1] == N0)
        indn = x + 1;
      return indn >= 0;
    }
    int i = (int)(x / g.ny), j = (int)(x % g.ny);
    if (i > 0 && m[x - g.ny] == N0)
      indn = x - g.ny;
    if (i < g.nx - 1 && m[x + g.ny] == N0)
      indn = x + g.ny;
    if (j > 0 && m[x - 1] == N0)
      indn = x - 1;
    if (j < g.ny - 1 && m[x + 1] == N0)
      indn = x + 1;
    return indn >= 0;
  }
};

// One layer.  In the reference's sweep a new cell copies the cell one step
// towards the interface along its normal if that cell's mask is >= 1 at
// that moment, else the layer-N0 neighbour it was reached from; cells of
// this layer visited earlier in the sweep already hold their copies, so a
// copy from one of them is followed to where it copied from.
template <int V>
__global__ void k_layer(double *__restrict__ grid, const int32_t *__restrict__ mprev,
                        int32_t *__restrict__ mnext, const double *__restrict__ dphi, Grid g,
                        int N0, int *__restrict__ err, const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= g.ncell)
    return;
  Layer Ly{mprev, g, N0};
  long indn;
  if (!Ly.in(c, indn)) {
    mnext[c] = mprev[c];
    return;
  }
  mnext[c] = mprev[c] == -2 ? -2 : N0 + 1;  // isolated cells return to -2
  long x = c, xn = indn, src = -1;
  for (int hops = 0; hops < 4096; hops++) {
    double n[2];
    long nind = -1;
    if (unit_normal(dphi, x, g.nd, n)) {
      int i = g.nd == 1 ? (int)x : (int)(x / g.ny), j = g.nd == 1 ? 0 : (int)(x % g.ny);
      int ind2[2] = {i, j}, ni[2] = {0, 0};
      for (int k = 0; k < g.nd; k++) {
        double h = k == 0 ? g.dx : g.dy;
        double xc = mul(add((double)ind2[k], 0.5), h);
        ni[k] = (int)dvd(sub(xc, mul(h, n[k])), h);
      }
      nind = g.nd == 1 ? ni[0] : (long)ni[0] * g.ny + ni[1];
    }
    bool off = nind < 0 || nind >= g.ncell;
    if (off) {
      atomicAdd(&err[2], 1);
      src = xn;
      break;
    }
    if (nind == x) {  // copies itself: keeps its own value
      src = x;
      break;
    }
    long nn;
    if (nind < x && Ly.in(nind, nn)) {  // filled earlier in this layer
      x = nind;
      xn = nn;
      continue;
    }
    src = mprev[nind] >= 1 ? nind : xn;
    break;
  }
  if (src < 0) {
    atomicAdd(&err[2], 1);
    return;
  }
  if (src != c)
    for (int v = 0; v < V - 1; v++)
      grid[c * V + v] = grid[src * V + v];
}

// Update mask of material mat (fill.cpp:364-365).
__global__ void k_mat_mask(const double *__restrict__ phi, const int32_t *__restrict__ im,
                           uint8_t *__restrict__ mask, long ncell,
                           const double *__restrict__ clk) {
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  int m = im[c];
  mask[c] = (phi[c] <= 0.0 && m != -2) || m == 1;
}

// ===========================================================================
// Merge, CFL and renormalisation over material grids.

// make_u (solvers/iterator.cpp:12-42): the level set averaged over the
// grids that updated the cell, the rest of the state from the grid of the
// cell's material (zero for a vacuum).
template <int V>
__global__ void k_make_u(double *__restrict__ u, const double *__restrict__ grids,
                         const uint8_t *__restrict__ masks, long ncell, int nmat, int eos0,
                         int eos1, const double *__restrict__ dt_dev) {
  if (dt_dev && *dt_dev == 0.0)
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  double s = 0.0, cnt = 0.0;
  for (int m = 0; m < nmat; m++)
    if (masks[(long)m * ncell + c]) {
      s += grids[((long)m * ncell + c) * V + V - 1];
      cnt += 1.0;
    }
  if (cnt > 0.0)
    u[c * V + V - 1] = s / cnt;
  int mi = u[c * V + V - 1] >= 0.0 ? 1 : 0;
  int eos = mi == 0 ? eos0 : eos1;
  for (int v = 0; v < V - 1; v++)
    u[c * V + v] = eos > -1 ? grids[((long)mi * ncell + c) * V + v] : 0.0;
}

// timestep (solvers/iterator.cpp:54-83): max over the masked cells of one
// material grid, accumulated over materials in *out.
template <class L>
__global__ void __launch_bounds__(256)
    k_cfl_max_masked(const double *__restrict__ u, const uint8_t *__restrict__ mask, long ncell,
                     int nd, double dx, double dy, unsigned long long *__restrict__ out,
                     DevPar P, const double *__restrict__ clk) {
  constexpr int V = L::V;
  if (clk && clk[0] >= clk[2])
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  double m = 0.0;
  if (c < ncell && mask[c]) {
    double q[V];
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

// renorm_distortion (solvers/utils.cpp:6-23) with each cell's material
// from its level set.
template <int V>
__global__ void k_renorm_multi(double *__restrict__ u, long ncell, double r00, double r01,
                               int eos0, int eos1, const double *__restrict__ dt_dev) {
  if (dt_dev && *dt_dev == 0.0)
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  double *q = u + c * V;
  int mi = q[V - 1] >= 0.0 ? 1 : 0;
  if ((mi == 0 ? eos0 : eos1) <= -1)
    return;
  double r = q[0];
  if (r > 0) {
    double A[9];
    for (int k = 0; k < 9; k++)
      A[k] = q[5 + k];
    double f = cbrt(r / ((mi == 0 ? r00 : r01) * det3(A)));
    for (int k = 0; k < 9; k++)
      q[5 + k] = A[k] * f;
  }
}

// Pointwise left_star_state for tests and the system.multi binding.
template <int V>
__global__ void k_star_pointwise(const double *__restrict__ QL, const double *__restrict__ QR,
                                 const double *__restrict__ nrm, double *__restrict__ out,
                                 long count, int nd, double dt, DevPar PL, DevPar PR) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= count)
    return;
  double n[2] = {nrm[k * nd], nd == 2 ? nrm[k * nd + 1] : 0.0};
  left_star_state(QL + k * V, QR + k * V, PL, PR, dt, n, nd, out + k * V);
}

}  // namespace multi
}  // namespace gpr
