// gpr_ops.cuh - host-side stage launchers of the GPR step, templated on the
// state layout (Layout<THERMAL, LSET>).  Every C ABI translation unit that
// serves a layout instantiates Ops<L> for it: gpr_capi.cu for V = 17 and
// V = 14, gpr_multi.cu for V = 15 (viscous, one level set).
#pragma once

#include "gpr_host.cuh"
#include "gpr_ode.cuh"
#include "gpr_osher.cuh"

namespace gpr {
namespace host {

// Pointwise kernels (one thread per state) behind gpr_flux / gpr_source /
// gpr_Bdot / gpr_max_abs_eigs / gpr_interface_terms.
template <class L>
__global__ void k_pointwise(int what, const double *__restrict__ Q, const double *__restrict__ X,
                            double *__restrict__ out, double *__restrict__ out2, long count,
                            int d, int flux, DevPar P, Consts C) {
  constexpr int V = L::V;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= count)
    return;
  double q[V], r[V];
#pragma unroll
  for (int k = 0; k < V; k++)
    q[k] = Q[c * V + k];
  Prim<L::THERMAL> s;
  prim<L::THERMAL>(q, P, s);
  switch (what) {
  case 0:  // flux (adds)
#pragma unroll
    for (int k = 0; k < V; k++)
      r[k] = out[c * V + k];
    flux_add<L::THERMAL, V>(q, s, d, P, r);
    break;
  case 1:
    source<L::THERMAL, V>(q, s, P, r);
    break;
  case 2: {
    double x[V];
#pragma unroll
    for (int k = 0; k < V; k++)
      x[k] = X[c * V + k];
    bdot<V, L::LSET>(s.v, x, d, r);
  } break;
  case 3:
    out[c] = max_abs_eigs<L::THERMAL>(q, s, d, P);
    return;
  case 5: {  // system_matrix along d through the x form (axis_swap)
    double pq[V], M[V * V];
#pragma unroll
    for (int k = 0; k < V; k++)
      pq[k] = q[axis_swap<L>(k, d)];
    Prim<L::THERMAL> ps;
    prim<L::THERMAL>(pq, P, ps);
    system_matrix<L::THERMAL, V>(pq, ps, P, M);
    for (int a = 0; a < V; a++)
      for (int b = 0; b < V; b++)
        out[(c * V + a) * V + b] = M[axis_swap<L>(a, d) * V + axis_swap<L>(b, d)];
    return;
  }
  case 6: {  // thermo_acoustic_tensor: Xi1 Xi2 along d
    constexpr int m = L::THERMAL ? 4 : 3;
    double X[m * m], l2;
    max_abs_eigs<L::THERMAL>(q, s, d, P, X, &l2);
#pragma unroll
    for (int e = 0; e < m * m; e++)
      out[c * m * m + e] = X[e];
    return;
  }
  default: {
    double qr[V], b[V];
#pragma unroll
    for (int k = 0; k < V; k++)
      qr[k] = X[c * V + k];
    if (flux == GPR_FLUX_RUSANOV)
      interface_point<L>(q, qr, d, P, C, r, b);
    else
      interface_point_eig<L>(q, qr, flux, P, C, r, b, d);
#pragma unroll
    for (int k = 0; k < V; k++)
      out2[c * V + k] = b[k];
  } break;
  }
#pragma unroll
  for (int k = 0; k < V; k++)
    out[c * V + k] = r[k];
}

// contorted (solvers/utils.cpp:66-85): raises *flag if a cell's normalised
// distortion has m0 - 1 > tol, where m0 = |A|_F^2 / (3 |det A|^(2/3)) (the
// mean over the singular values s_i of s_i^2 / det^(2/3), without the SVD).
// Skipped when the device clock says the step did not run (dt == 0).
template <int V>
__global__ void k_contorted(const double *__restrict__ u, long ncell, double tol,
                            int *__restrict__ flag, const double *__restrict__ dt_dev) {
  if (dt_dev && *dt_dev == 0.0)
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  const double *A = u + c * V + 5;
  double f2 = 0.0;
#pragma unroll
  for (int k = 0; k < 9; k++)
    f2 += A[k] * A[k];
  double d13 = cbrt(fabs(det3(A)));
  if (f2 / (3.0 * d13 * d13) - 1.0 > tol)
    atomicOr(flag, 1);
}

// reset_distortion (solvers/utils.cpp:44-64) when *flag is set: every cell
// of a non-vacuum material loses its distortion energy rho E_2A and gets
// A = (rho / rho0)^(1/3) I.  The material is 0, or that of the level set
// (functions/vectors.cpp:24-31) with one.
template <class L>
__global__ void k_reset_distortion(double *__restrict__ u, long ncell,
                                   const int *__restrict__ flag, DevPar P0, DevPar P1,
                                   const double *__restrict__ dt_dev) {
  constexpr int V = L::V;
  if (!*flag || (dt_dev && *dt_dev == 0.0))
    return;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  double *q = u + c * V;
  int mi = L::LSET > 0 && q[V - 1] >= 0.0 ? 1 : 0;
  const DevPar &P = mi ? P1 : P0;
  if (P.EOS <= -1)
    return;
  double r = q[0], ir = 1.0 / r;
  const double *A = q + 5;
  // E_2A = C_0 / 4 |dev(A A^T)|^2 (energy/eos.cpp, functions/matrices.cpp:16-26)
  double G00 = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  double G11 = A[3] * A[3] + A[4] * A[4] + A[5] * A[5];
  double G22 = A[6] * A[6] + A[7] * A[7] + A[8] * A[8];
  double G01 = A[0] * A[3] + A[1] * A[4] + A[2] * A[5];
  double G02 = A[0] * A[6] + A[1] * A[7] + A[2] * A[8];
  double G12 = A[3] * A[6] + A[4] * A[7] + A[5] * A[8];
  double t = (G00 + G11 + G22) / 3.0;
  double dg = (G00 - t) * (G00 - t) + (G11 - t) * (G11 - t) + (G22 - t) * (G22 - t) +
              2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
  double Gm = eos_rho(r, ir, P).G;
  double cs2 = P.beta == 0.0 ? P.b02 : P.b02 * pow(r * P.ir0, P.beta);
  double C0 = (1.0 - P.beta / Gm) * cs2;
  q[1] -= r * (C0 / 4.0 * dg);
  double cc = cbrt(r * P.ir0);
#pragma unroll
  for (int k = 0; k < 9; k++)
    q[5 + k] = (k % 4) == 0 ? cc : 0.0;
}

template <class L> struct Ops {
  static constexpr int V = L::V;

  static int boundaries(const double *u, double *ub, const int32_t *nX, int nd,
                        const int32_t *bcs, cudaStream_t st) {
    int nx = nX[0], ny = nd == 2 ? nX[1] : 1;
    if (nd == 1) {
      k_boundaries1d<V><<<blocks((long)(nx + 2 * NN) * V, 256), 256, 0, st>>>(u, ub, nx, bcs[0],
                                                                              bcs[1]);
      return cuda_rc();
    }
    long n = (long)nx * ny * V;
    k_fill_interior<V><<<blocks(n, 256), 256, 0, st>>>(u, ub, nx, ny, nd);
    long g0 = (long)(nd == 1 ? 1 : ny) * 2 * NN * V;
    k_ghosts<V><<<blocks(g0, 256), 256, 0, st>>>(ub, nx, ny, nd, 0, bcs[0], bcs[1]);
    if (nd == 2) {
      long g1 = (long)(nx + 2 * NN) * 2 * NN * V;
      k_ghosts<V><<<blocks(g1, 256), 256, 0, st>>>(ub, nx, ny, nd, 1, bcs[2], bcs[3]);
    }
    return cuda_rc();
  }

  static long weno_scratch(const int32_t *nX, int nd) {
    if (nd == 1)
      return 0;
    return (long)(nX[0] + 2) * (nX[1] + 2 * NN) * NN * V;
  }

  static int weno(double *wh, const double *ub, const int32_t *nX, int nd, double *scratch,
                  cudaStream_t st) {
    const Consts &C = consts();
    if (nd == 1) {
      int ncb = nX[0] + 2;
      k_weno1d<V><<<GPR_SPREAD((long)ncb * V, 256), 0, st>>>(wh, ub, ncb, C);
      return cuda_rc();
    }
    // both sweeps in one launch through shared memory (k_weno2d); the
    // scratch is not used
    int nxp = nX[0] + 2, nyp = nX[1] + 2;
    const int tj = weno2d_tile(nyp);
    const long nblk = (long)nxp * ((nyp + tj - 1) / tj);
    k_weno2d<V><<<(unsigned)nblk, WENO2_THREADS, 0, st>>>(wh, ub, nxp, nyp, tj, C);
    return cuda_rc();
  }

  // Deferred Picard cells (PicardResume) in a caller's scratch of at least
  // predictor_resume_doubles(ncb) doubles: the list, its length, the next
  // iteration indices and the smallest updates.
  static long predictor_resume_doubles(long ncb) { return 2 * ncb + 8; }
  static PicardResume resume_view(double *scr, long ncb) {
    PicardResume R;
    R.cap = 3;
    R.dmin = scr;
    R.it = (int *)(scr + ncb);
    R.list = R.it + ncb;
    R.n = R.list + ncb;
    return R;
  }

  // resume: optional scratch (predictor_resume_doubles) with which, on grids
  // of 8192 cells or more, cells still iterating after three Picard
  // iterations continue in a second launch over a compacted list of them
  // (k_predictor_picard, PicardResume).
  static int predictor(double *qh, const double *wh, double dt, const double *dt_dev,
                       const double *dX, int nd, const int32_t *nX, int stiff,
                       const DevPar &P, const uint8_t *mask, int32_t *status,
                       cudaStream_t st, double *resume = nullptr) {
    const Consts &C = consts();
    long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
    double idx = 1.0 / dX[0], idy = nd == 2 ? 1.0 / dX[1] : 1.0;
    // the first Picard iterate at one thread per spatial node (k_predictor_first)
    const int first = stiff ? 0 : 1;
    PicardResume R, R2;
    // Below ~8k cells the Picard launch fits in one wave of resident warps,
    // so there are no later warps to free and the continuation would only
    // add its launch (the 200-cell tube: ~8 us per step).
    if (resume && !stiff && ncb >= 8192) {
      R = resume_view(resume, ncb);
      cudaMemsetAsync(R.n, 0, sizeof(int), st);
      R2.it = R.it;
      R2.dmin = R.dmin;
      R2.in = R.list;
      R2.n_in = R.n;
    }
    if (nd == 1) {
      if (first)
        k_predictor_first<L, 1><<<GPR_SPREAD(ncb * NN, 128), 0, st>>>(
            qh, wh, ncb, mask, dt, dt_dev, idx, idy, P, C, Batch{});
      long nt = ncb * NN * NN;
      k_predictor_picard<L, 1><<<GPR_SPREAD(nt, 128), 0, st>>>(
          qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, stiff, P, C, Batch{}, first, R);
      if (R.cap)
        k_predictor_picard<L, 1><<<GPR_SPREAD(nt, 128), 0, st>>>(
            qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, stiff, P, C, Batch{}, first, R2);
      return stiff_pass<1>(qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, P, C, st);
    }
    if (first)
      k_predictor_first<L, 2><<<GPR_SPREAD(ncb * NN * NN, 128), 0, st>>>(
          qh, wh, ncb, mask, dt, dt_dev, idx, idy, P, C, Batch{});
    long nt = ncb * NN * NN * NN;
    k_predictor_picard<L, 2><<<GPR_SPREAD(nt, 128), 0, st>>>(
        qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, stiff, P, C, Batch{}, first, R);
    if (R.cap)
      k_predictor_picard<L, 2><<<GPR_SPREAD(nt, 128), 0, st>>>(
          qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, stiff, P, C, Batch{}, first, R2);
    return stiff_pass<2>(qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, P, C, st);
  }

  // Stiff-source Newton pass over the cells the Picard pass flagged.
  template <int ND, bool BATCH = false>
  static int stiff_pass(double *qh, const double *wh, long ncb, const uint8_t *mask,
                        int32_t *status, double dt, const double *dt_dev, double idx,
                        double idy, const DevPar &P, const Consts &C, cudaStream_t st,
                        const Batch &B = Batch{}) {
    return launch_stiff<L, ND, BATCH>(qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, P, C,
                                      st, B);
  }

  static long fv_scratch(const int32_t *nX, int nd) {
    if (nd == 1)
      return (long)(nX[0] + 1) * 2 * V;
    // x and y face sums, then the per-point terms of one direction (Osher /
    // Roe, k_faces2d_eigp)
    const long nf = (long)(nX[0] + 1) * (nX[1] + 1);
    return 2L * nf * 2 * V + nf * NN * NN * 2 * V;
  }

  // parts: FV_BOTH (fv_launcher), FV_CENTERS (centers1/2: the volume term,
  // no scratch needed) or FV_INTERFS (interfs1/2: the face terms).
  static int fv(double *u, const double *qh, const int32_t *nX, double dt,
                const double *dt_dev, const double *dX, int nd, int sources, int time_dg,
                const DevPar &P, const uint8_t *mask, double *scratch, cudaStream_t st,
                int flux = GPR_FLUX_RUSANOV, int parts = FV_BOTH) {
    const Consts &C = consts();
    int nx = nX[0];
    const bool faces = parts & FV_INTERFS;
    if (nd == 1) {
      if (flux == GPR_FLUX_RUSANOV || !faces) {
        // faces, volume term and update in one launch (k_fv1d)
        if (blocks(nx, FV1_TILE) < 2 * sm_count())
          k_fv1d<L, FV1_TILE_SMALL><<<blocks(nx, FV1_TILE_SMALL), 4 * (FV1_TILE_SMALL + 1), 0,
                                      st>>>(u, qh, nx, mask, dt, dt_dev, dX[0], sources,
                                            time_dg, P, C, parts);
        else
          k_fv1d<L><<<blocks(nx, FV1_TILE), 128, 0, st>>>(u, qh, nx, mask, dt, dt_dev, dX[0],
                                                          sources, time_dg, P, C, parts);
        return cuda_rc();
      }
      // Osher / Roe: the faces' eigen-decompositions, one warp each, write
      // the face sums to scratch (a 1D grid has few faces, so one launch over
      // all of them keeps the decompositions' latency to one), then the cell
      // pass applies them
      k_faces1d_eigw<L><<<(unsigned)(nx + 1), 32 * EIG_WARPS, 0, st>>>(
          scratch, qh, (long)nx + 1, mask, dt, dt_dev, dX[0], time_dg, flux, P, C, Batch{});
      long nc = (long)nx * NN * NN;
      k_cells<L, 1><<<GPR_SPREAD(nc, 128), 0, st>>>(u, qh, scratch, nullptr, nx, 1, mask, dt,
                                                     dt_dev, dX[0], 1.0, sources, time_dg, P,
                                                     C, Batch{}, parts);
      return cuda_rc();
    }
    int ny = nX[1];
    const long nc = (long)nx * ny * NN * NN * NN;
    if (flux == GPR_FLUX_RUSANOV || !faces) {
      // Rusanov: the volume term first (centers2), then the face terms
      // applied to u in place by four passes (x / y faces, even / odd index
      // along the direction; two faces of one pass never share a cell), as
      // interfs2 updates u inside its face loop (fv.cpp:162-279).  No face
      // buffer.
      if (parts & FV_CENTERS)
        k_cells<L, 2><<<blocks(nc, 128), 128, 0, st>>>(u, qh, nullptr, nullptr, nx, ny, mask,
                                                        dt, dt_dev, dX[0], dX[1], sources,
                                                        time_dg, P, C, Batch{}, FV_CENTERS);
      if (faces)
        for (int dir = 0; dir < 2; dir++)
          for (int par = 0; par < 2; par++) {
            long nf = face2_count(nx, ny, dir, par);
            k_faces2d<L><<<blocks(nf * NN * NN, 128), 128, 0, st>>>(
                u, qh, nx, ny, dir, mask, dt, dt_dev, dX[0], dX[1], time_dg, P, C, par);
          }
      return cuda_rc();
    }
    // Osher / Roe: the per-thread eigen-decompositions write the face sums
    // of each direction to scratch, then the cell pass applies the volume
    // and face terms
    long nf = (long)(nx + 1) * (ny + 1);
    double *fbx = scratch, *fby = scratch + nf * 2 * V, *pp = scratch + 2 * nf * 2 * V;
    faces2d_eig(fbx, pp, qh, nx, ny, 0, mask, dt, dt_dev, dX, time_dg, flux, P, C, st);
    faces2d_eig(fby, pp, qh, nx, ny, 1, mask, dt, dt_dev, dX, time_dg, flux, P, C, st);
    k_cells<L, 2><<<blocks(nc, 128), 128, 0, st>>>(u, qh, fbx, fby, nx, ny, mask, dt, dt_dev,
                                                    dX[0], dX[1], sources, time_dg, P, C,
                                                    Batch{}, parts);
    return cuda_rc();
  }

  // Face pass of the FV update only: the k_faces kernels writing the face
  // contributions (to the left and right cells) into fb.
  static int faces(const double *qh, const int32_t *nX, double dt, const double *dX, int nd,
                   int time_dg, const DevPar &P, const uint8_t *mask, double *fb,
                   cudaStream_t st, int flux = GPR_FLUX_RUSANOV) {
    const Consts &C = consts();
    int nx = nX[0];
    if (nd == 1) {
      long nf = (long)(nx + 1) * NN;
      if (flux == GPR_FLUX_RUSANOV)
        k_faces1d_split<L><<<GPR_SPREAD(nf * 2, 128), 0, st>>>(
            fb, qh, (long)nx + 1, mask, dt, nullptr, dX[0], time_dg, P, C, Batch{});
      else
        k_faces1d_eigw<L><<<(unsigned)(nx + 1), 32 * EIG_WARPS, 0, st>>>(
            fb, qh, (long)nx + 1, mask, dt, nullptr, dX[0], time_dg, flux, P, C, Batch{});
      return cuda_rc();
    }
    int ny = nX[1];
    long nf = (long)(nx + 1) * (ny + 1);
    if (flux != GPR_FLUX_RUSANOV) {
      double *pp = fb + 2 * nf * 2 * V;
      faces2d_eig(fb, pp, qh, nx, ny, 0, mask, dt, nullptr, dX, time_dg, flux, P, C, st);
      faces2d_eig(fb + nf * 2 * V, pp, qh, nx, ny, 1, mask, dt, nullptr, dX, time_dg, flux, P,
                  C, st);
      return cuda_rc();
    }
    k_faces2d<L><<<blocks(nf * NN * NN, 128), 128, 0, st>>>(fb, qh, nx, ny, 0, mask, dt,
                                                             nullptr, dX[0], dX[1], time_dg,
                                                             P, C);
    k_faces2d<L><<<blocks(nf * NN * NN, 128), 128, 0, st>>>(fb + nf * 2 * V, qh, nx, ny, 1,
                                                             mask, dt, nullptr, dX[0], dX[1],
                                                             time_dg, P, C);
    return cuda_rc();
  }

  // Osher / Roe faces of one direction on a 2D grid: one thread per face
  // quadrature point into the per-point buffer pp (nf x 4 x 2V doubles),
  // then the face sums into fb.
  static void faces2d_eig(double *fb, double *pp, const double *qh, int nx, int ny, int dir,
                          const uint8_t *mask, double dt, const double *dt_dev, const double *dX,
                          int time_dg, int flux, const DevPar &P, const Consts &C,
                          cudaStream_t st) {
    long nf = (long)(nx + 1) * (ny + 1);
    k_faces2d_eigp<L><<<blocks(nf * NN * NN, 64), 64, 0, st>>>(
        pp, qh, nx, ny, dir, mask, dt, dt_dev, dX[0], dX[1], time_dg, flux, P, C);
    k_faces2d_eigsum<V><<<blocks(nf * 2 * V, 256), 256, 0, st>>>(fb, pp, nf);
  }

  static int timestep(const double *u, long ncell, const double *dX, int nd, double cfl,
                      double t, double tf, int count, const DevPar &P, double *dt_out,
                      double *scratch, cudaStream_t st) {
    unsigned long long *mx = (unsigned long long *)scratch;
    cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st);
    k_cfl_max<L><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, nd, dX[0],
                                                      nd == 2 ? dX[1] : 1.0, mx, P);
    k_cfl_finalize<<<1, 1, 0, st>>>(mx, cfl, t, tf, count, dt_out);
    return cuda_rc();
  }

  static int renorm(double *u, long ncell, const DevPar &P, cudaStream_t st) {
    k_renorm<V><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, P.rho0, nullptr);
    return cuda_rc();
  }

  // contorted + reset_distortion after a step (iterator.cpp:150-151); flag
  // is device scratch for one int.
  static void contortion(double *u, long ncell, double tol, const DevPar &P0, const DevPar &P1,
                         int *flag, const double *dt_dev, cudaStream_t st) {
    cudaMemsetAsync(flag, 0, sizeof(int), st);
    k_contorted<V><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, tol, flag, dt_dev);
    k_reset_distortion<L><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, flag, P0, P1, dt_dev);
  }

  static int pointwise(int what, const double *Q, const double *X, double *out, double *out2,
                       long count, int d, int flux, const DevPar &P, cudaStream_t st) {
    k_pointwise<L><<<blocks(count, 64), 64, 0, st>>>(what, Q, X, out, out2, count, d, flux, P,
                                                     consts());
    return cuda_rc();
  }

  // One device-resident iterator step (iterator.cpp:119-151 for one
  // material): CFL -> boundaries -> WENO -> predictor -> FV -> renorm ->
  // clock advance, with dt living in clk[1].
  static int iterate(double *u, const int32_t *nX, int nd, const double *dX,
                     const int32_t *bcs, const DevPar &P, const uint8_t *mask, double *clk,
                     int nsteps, double *scratch, int32_t *status, cudaStream_t st,
                     int flux = GPR_FLUX_RUSANOV, double contorted_tol = INFINITY) {
    long ncell = nd == 1 ? nX[0] : (long)nX[0] * nX[1];
    long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
    long nub = nd == 1 ? nX[0] + 2 * NN : (long)(nX[0] + 2 * NN) * (nX[1] + 2 * NN);
    long ns = nd == 1 ? NN : NN * NN;
    double *ub = scratch;
    double *wh = ub + nub * V;
    double *qh = wh + ncb * ns * V;
    double *tmp = qh + ncb * NN * ns * V;
    unsigned long long *mx = (unsigned long long *)(tmp + (weno_scratch(nX, nd) > fv_scratch(nX, nd)
                                                               ? weno_scratch(nX, nd)
                                                               : fv_scratch(nX, nd)));
    double *dt_dev = clk + 1;
    if (nsteps > 0)
      cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), st);
    for (int s = 0; s < nsteps; s++) {
      step_head(u, ncell, nd, dX, P, mx, clk, st);
      int rc = boundaries(u, ub, nX, nd, bcs, st);
      if (rc)
        return rc;
      rc = weno(wh, ub, nX, nd, tmp, st);
      if (rc)
        return rc;
      // tmp (the FV face buffers, used after the predictor) holds the
      // predictor's deferred cells meanwhile
      rc = predictor(qh, wh, 0.0, dt_dev, dX, nd, nX, 0, P, mask, status, st, tmp);
      if (rc)
        return rc;
      rc = fv(u, qh, nX, 0.0, dt_dev, dX, nd, 1, 1, P, mask, tmp, st, flux);
      if (rc)
        return rc;
      step_tail(u, ncell, P, contorted_tol, mx, clk, st);
    }
    return cuda_rc();
  }

  // The clock kernels of a device-resident step around its stages:
  // head = CFL maximum -> dt (and the contortion flag mx[1] cleared); tail =
  // renorm + contortion test -> reset -> clock advance (and the CFL maximum
  // mx[0] cleared for the next step).  mx[0..1] must be zero before the
  // first step.
  static void step_head(const double *u, long ncell, int nd, const double *dX, const DevPar &P,
                        unsigned long long *mx, double *clk, cudaStream_t st) {
    k_cfl_max<L><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, nd, dX[0],
                                                      nd == 2 ? dX[1] : 1.0, mx, P);
    k_clock_finalize<<<1, 1, 0, st>>>(mx, clk, (int *)(mx + 1));
  }
  static void step_tail(double *u, long ncell, const DevPar &P, double tol,
                        unsigned long long *mx, double *clk, cudaStream_t st) {
    const double *dt_dev = clk + 1;
    int *flag = (int *)(mx + 1);
    k_renorm_contorted<V><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, P.rho0, tol, flag,
                                                               dt_dev);
    k_reset_distortion<L><<<GPR_SPREAD(ncell, 256), 0, st>>>(u, ncell, flag, P, P, dt_dev);
    k_clock_advance<<<1, 1, 0, st>>>(clk, mx);
  }

  // ---- split scheme (steppers.cpp:50-66, split/homogeneous.cpp) -------------
  static int midstep(double *wh, double dt, const double *dt_dev, const double *dX, int nd,
                     const int32_t *nX, const DevPar &P, const uint8_t *mask, cudaStream_t st) {
    const Consts &C = consts();
    long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
    double idx = 1.0 / dX[0], idy = nd == 2 ? 1.0 / dX[1] : 1.0;
    if (nd == 1)
      k_midstep<L, 1><<<GPR_SPREAD(ncb * NN, 128), 0, st>>>(wh, ncb, mask, dt, dt_dev, idx,
                                                              idy, P, C);
    else
      k_midstep<L, 2><<<GPR_SPREAD(ncb * NN * NN, 128), 0, st>>>(wh, ncb, mask, dt, dt_dev,
                                                                   idx, idy, P, C);
    return cuda_rc();
  }

  // ODE half step on u and ub, WENO, [midstepper], FV without sources and
  // time integration on the node values, ODE half step on u; ub is modified.
  // scratch: wh then the WENO / FV temporary.
  static int split_stepper(double *u, double *ub, const int32_t *nX, int nd, double dt,
                           const double *dt_dev, const double *dX, int half_step, int flux,
                           const DevPar &P, const uint8_t *mask, double *scratch,
                           cudaStream_t st) {
    long ncell = nd == 1 ? nX[0] : (long)nX[0] * nX[1];
    long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
    long nub = nd == 1 ? nX[0] + 2 * NN : (long)(nX[0] + 2 * NN) * (nX[1] + 2 * NN);
    long ns = nd == 1 ? NN : NN * NN;
    double *wh = scratch, *tmp = wh + ncb * ns * V;
    // the half steps on u and ub in one launch
    k_ode<L><<<GPR_SPREAD(ncell + nub, 128), 0, st>>>(u, ncell, dt / 2, dt_dev, 0.5, P, ub,
                                                       nub);
    int rc = weno(wh, ub, nX, nd, tmp, st);
    if (rc)
      return rc;
    if (half_step && (rc = midstep(wh, dt, dt_dev, dX, nd, nX, P, mask, st)))
      return rc;
    rc = fv(u, wh, nX, dt, dt_dev, dX, nd, 0, 0, P, mask, tmp, st, flux);
    if (rc)
      return rc;
    k_ode<L><<<GPR_SPREAD(ncell, 128), 0, st>>>(u, ncell, dt / 2, dt_dev, 0.5, P);
    return cuda_rc();
  }

  static long split_scratch(const int32_t *nX, int nd) {
    long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
    long ns = nd == 1 ? NN : NN * NN;
    long w = weno_scratch(nX, nd), f = fv_scratch(nX, nd);
    return ncb * ns * V + (w > f ? w : f);
  }

  // Device-resident iterator with the split scheme (iterator.cpp:109-151,
  // SPLIT = true); scratch as iterate().
  static int iterate_split(double *u, const int32_t *nX, int nd, const double *dX,
                           const int32_t *bcs, const DevPar &P, const uint8_t *mask,
                           double *clk, int nsteps, double *scratch, int half_step, int flux,
                           cudaStream_t st, double contorted_tol = INFINITY) {
    long ncell = nd == 1 ? nX[0] : (long)nX[0] * nX[1];
    long nub = nd == 1 ? nX[0] + 2 * NN : (long)(nX[0] + 2 * NN) * (nX[1] + 2 * NN);
    double *ub = scratch;
    double *rest = ub + nub * V;
    unsigned long long *mx = (unsigned long long *)(scratch + iterate_scratch(nX, nd) - 2);
    double *dt_dev = clk + 1;
    if (nsteps > 0)
      cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), st);
    for (int s = 0; s < nsteps; s++) {
      step_head(u, ncell, nd, dX, P, mx, clk, st);
      int rc = boundaries(u, ub, nX, nd, bcs, st);
      if (rc)
        return rc;
      rc = split_stepper(u, ub, nX, nd, 0.0, dt_dev, dX, half_step, flux, P, mask, rest, st);
      if (rc)
        return rc;
      step_tail(u, ncell, P, contorted_tol, mx, clk, st);
    }
    return cuda_rc();
  }

  static long iterate_scratch(const int32_t *nX, int nd) {
    long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
    long nub = nd == 1 ? nX[0] + 2 * NN : (long)(nX[0] + 2 * NN) * (nX[1] + 2 * NN);
    long ns = nd == 1 ? NN : NN * NN;
    long w = weno_scratch(nX, nd), f = fv_scratch(nX, nd);
    // + the CFL maximum and the contortion flag
    return nub * V + ncb * ns * V + ncb * NN * ns * V + (w > f ? w : f) + 2;
  }

  // ---- batched form -------------------------------------------------------
  static BatchLayout batch_layout(int ninst, const int32_t *nx) {
    return batch_layout_v(ninst, nx, V);
  }

  static Batch batch_view(double *scr, int ninst, const BatchLayout &b, double *clk) {
    return batch_view_of(scr, ninst, b, clk);
  }

  // The stages of one batched step with the launch shapes sh.
  static void batch_cfl(double *u, unsigned long long *mx, const BatchLayout &b, const Batch &B,
                        int ninst, cudaStream_t st) {
    k_b_cfl_max<L><<<blocks(b.nu, 256), 256, 0, st>>>(u, b.nu, mx, B);
    k_b_clock_finalize<<<blocks(ninst, 128), 128, 0, st>>>(mx, B);
  }
  static void batch_weno(double *wh, const double *ub, const BatchLayout &b, const Batch &B,
                         int bs, cudaStream_t st) {
    k_b_weno<V><<<blocks(b.nb * V, bs), bs, 0, st>>>(wh, ub, b.nb, consts(), B);
  }
  static void batch_picard_pair(double *qh, const double *wh, int32_t *status,
                                const BatchLayout &b, const Batch &B, int bs_first,
                                int bs_picard, double *scr, cudaStream_t st) {
    const Consts &C = consts();
    DevPar P0{};
    PicardResume R;
    R.cap = 3;
    R.list = (int *)(scr + b.o_rlist);
    R.n = (int *)(scr + b.o_rn);
    R.it = (int *)(scr + b.o_rit);
    R.dmin = scr + b.o_rdmin;
    cudaMemsetAsync(R.n, 0, sizeof(int), st);
    k_predictor_first<L, 1, true><<<blocks(b.nb * NN, bs_first), bs_first, 0, st>>>(
        qh, wh, b.nb, nullptr, 0.0, nullptr, 1.0, 1.0, P0, C, B);
    k_predictor_picard<L, 1, true><<<blocks(b.nb * NN * NN, bs_picard), bs_picard, 0, st>>>(
        qh, wh, b.nb, nullptr, status, 0.0, nullptr, 1.0, 1.0, 0, P0, C, B, 1, R);
    PicardResume R2;
    R2.it = R.it;
    R2.dmin = R.dmin;
    R2.in = R.list;
    R2.n_in = R.n;
    k_predictor_picard<L, 1, true><<<blocks(b.nb * NN * NN, bs_picard), bs_picard, 0, st>>>(
        qh, wh, b.nb, nullptr, status, 0.0, nullptr, 1.0, 1.0, 0, P0, C, B, 1, R2);
  }
  static void batch_faces(double *fb, const double *qh, const BatchLayout &b, const Batch &B,
                          int split, int bs, cudaStream_t st) {
    const Consts &C = consts();
    DevPar P0{};
    if (split)
      k_faces1d_split<L, true><<<blocks(b.nf * NN * 2, bs), bs, 0, st>>>(
          fb, qh, b.nf, nullptr, 0.0, nullptr, 1.0, 1, P0, C, B);
    else
      k_faces1d<L, true><<<blocks(b.nf * NN, bs), bs, 0, st>>>(fb, qh, b.nf, nullptr, 0.0,
                                                                nullptr, 1.0, 1, P0, C, B);
  }
  static void batch_cells(double *u, const double *qh, const double *fb, const BatchLayout &b,
                          const Batch &B, int bs, cudaStream_t st) {
    DevPar P0{};
    k_cells<L, 1, true><<<blocks(b.nu * NN * NN, bs), bs, 0, st>>>(
        u, qh, fb, nullptr, b.nu, 1, nullptr, 0.0, nullptr, 1.0, 1.0, 1, 1, P0, consts(), B,
        FV_BOTH);
  }

  static int batch_iterate(double *u, double *clk, int ninst, const int32_t *nx, int nsteps,
                           double *scr, int32_t *status, unsigned long long *updates,
                           cudaStream_t st, const BatchShapes &sh = BatchShapes{}) {
    const Consts &C = consts();
    BatchLayout b = batch_layout(ninst, nx);
    Batch B = batch_view(scr, ninst, b, clk);
    double *ub = scr + b.o_ub, *wh = scr + b.o_wh, *qh = scr + b.o_qh, *fb = scr + b.o_fb;
    unsigned long long *mx = (unsigned long long *)(scr + b.o_mx);
    DevPar P0{};
    for (int s = 0; s < nsteps; s++) {
      batch_cfl(u, mx, b, B, ninst, st);
      k_b_boundaries<V><<<blocks(b.nub * V, 256), 256, 0, st>>>(u, ub, b.nub, B);
      batch_weno(wh, ub, b, B, sh.weno, st);
      batch_picard_pair(qh, wh, status, b, B, sh.first, sh.picard, scr, st);
      int rc = stiff_pass<1, true>(qh, wh, b.nb, nullptr, status, 0.0, nullptr, 1.0, 1.0, P0,
                                   C, st, B);
      if (rc)
        return rc;
      batch_faces(fb, qh, b, B, sh.faces_split, sh.faces, st);
      batch_cells(u, qh, fb, b, B, sh.cells, st);
      k_b_renorm<V><<<blocks(b.nu, 256), 256, 0, st>>>(u, b.nu, B);
      k_b_clock_advance<<<blocks(ninst, 128), 128, 0, st>>>(B, updates);
    }
    return cuda_rc();
  }

  // Autotuner of the batched step's launch shapes.  On the batch's current
  // state it times every candidate of each stage with CUDA events on the
  // stream (one untimed launch, then `reps` timed ones) and keeps the fastest
  // in sh: WENO at 64 / 128 / 256 / 512 threads per block; the predictor pair
  // (first iterate + Picard) at 32 / 64 / 128 threads per block each (8 to
  // 32 predictor cells per Picard block); the face pass in both lane layouts
  // (2 or 4 lanes per face) at 32 / 64 / 128; the volume pass at 32 / 64 /
  // 128.  Every timed launch is idempotent on what the step reads (ub -> wh,
  // wh -> qh, qh -> fb); the volume pass updates u in place, so it is timed
  // on a copy of u in the ub area.  Afterwards u is unchanged, each clock
  // holds this step's dt (as after the first kernels of a step) and ub, wh,
  // qh and fb hold intermediate values that the next step overwrites.
  // times[NCAND] (optional) receives the mean time in ms of each candidate,
  // in the order above (4 + 9 + 6 + 3).  Synchronises the stream.
  static constexpr int NCAND = 4 + 9 + 6 + 3;
  static int batch_autotune(double *u, double *clk, int ninst, const int32_t *nx, double *scr,
                            BatchShapes &sh, float *times, int reps, cudaStream_t st) {
    BatchLayout b = batch_layout(ninst, nx);
    Batch B = batch_view(scr, ninst, b, clk);
    double *ub = scr + b.o_ub, *wh = scr + b.o_wh, *qh = scr + b.o_qh, *fb = scr + b.o_fb;
    unsigned long long *mx = (unsigned long long *)(scr + b.o_mx);
    const Consts &C = consts();
    DevPar P0{};
    if (reps < 1)
      reps = 1;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess)
      return GPR_E_CUDA;
    if (cudaEventCreate(&e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      return GPR_E_CUDA;
    }
    int rc = GPR_OK;
    int slot = 0;
    // mean ms of `reps` runs of f after one untimed run; -1 on a CUDA error
    auto timeit = [&](auto f) -> float {
      f();
      cudaEventRecord(e0, st);
      for (int r = 0; r < reps; r++)
        f();
      cudaEventRecord(e1, st);
      float ms = -1.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) !=
                                                         cudaSuccess ||
          cudaGetLastError() != cudaSuccess) {
        rc = GPR_E_CUDA;
        return -1.f;
      }
      ms /= reps;
      if (times)
        times[slot] = ms;
      slot++;
      return ms;
    };
    const int bs3[3] = {32, 64, 128};
    // this step's dt and ghost cells
    batch_cfl(u, mx, b, B, ninst, st);
    k_b_boundaries<V><<<blocks(b.nub * V, 256), 256, 0, st>>>(u, ub, b.nub, B);
    {
      const int cand[4] = {64, 128, 256, 512};
      float best = 1e30f;
      for (int c : cand) {
        float ms = timeit([&] { batch_weno(wh, ub, b, B, c, st); });
        if (rc)
          break;
        if (ms < best) {
          best = ms;
          sh.weno = c;
        }
      }
    }
    if (!rc) {
      float best = 1e30f;
      for (int f : bs3)
        for (int p : bs3) {
          float ms = timeit([&] { batch_picard_pair(qh, wh, nullptr, b, B, f, p, scr, st); });
          if (rc)
            break;
          if (ms < best) {
            best = ms;
            sh.first = f;
            sh.picard = p;
          }
        }
    }
    if (!rc) {
      // a complete predictor (the Newton pass finishes flagged cells) for the
      // face and volume timings
      batch_picard_pair(qh, wh, nullptr, b, B, sh.first, sh.picard, scr, st);
      rc = stiff_pass<1, true>(qh, wh, b.nb, nullptr, nullptr, 0.0, nullptr, 1.0, 1.0, P0, C,
                               st, B);
    }
    if (!rc) {
      float best = 1e30f;
      for (int split = 0; split < 2 && !rc; split++)
        for (int c : bs3) {
          float ms = timeit([&] { batch_faces(fb, qh, b, B, split, c, st); });
          if (rc)
            break;
          if (ms < best) {
            best = ms;
            sh.faces_split = split;
            sh.faces = c;
          }
        }
    }
    if (!rc) {
      // the volume pass on a copy of u (ub holds nub >= nu cells)
      if (cudaMemcpyAsync(ub, u, sizeof(double) * b.nu * V, cudaMemcpyDeviceToDevice, st) !=
          cudaSuccess)
        rc = GPR_E_CUDA;
      float best = 1e30f;
      for (int c : bs3) {
        if (rc)
          break;
        float ms = timeit([&] { batch_cells(ub, qh, fb, b, B, c, st); });
        if (rc)
          break;
        if (ms < best) {
          best = ms;
          sh.cells = c;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc)
      fprintf(stderr, "gpr_gb300: batch autotune: CUDA error\n");
    return rc;
  }

  static int ode(double *u, long ncell, double dt, const DevPar &P, cudaStream_t st) {
    k_ode<L><<<GPR_SPREAD(ncell, 128), 0, st>>>(u, ncell, dt, nullptr, 1.0, P);
    return cuda_rc();
  }
};

using L17 = Layout<true, 0>;
using L14 = Layout<false, 0>;
using L15 = Layout<false, 1>;

}  // namespace host
}  // namespace gpr
