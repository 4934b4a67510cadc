// gpr_multi.cu - C ABI of the level-set ghost fluid (include/gpr_gb300.h,
// "ghost fluid") and the stage launchers of the V = 15 layout (viscous, one
// level set) that the dispatch of gpr_capi.cu forwards to.
//
// The fill of one call (fill_ghost_cells, multi/fill.cpp:330-370):
//   re-distance u's level set (k_fmm_*) and write it back into u;
//   per material: copy u into its grid, the material level set and its
//   normals, the interface cells, the boundary-cell plan, the star states
//   (level 0 in parallel, deeper levels in one block), their scatter, the
//   19 extrapolation layers and the update mask.
// Everything is stream-ordered and nothing synchronises; per-call error
// counts accumulate in the caller's status[4] (device int32):
//   [0] re-distancing did not converge within its round budget,
//   [1] boundary cells whose fill would read outside the grid in the
//       reference (left unfilled), [2] layer cells whose copy source would
//       lie outside the grid (they copy their layer neighbour instead),
//   [3] reserved.
#include <stdio.h>

#include "gpr_multi.cuh"
#include "gpr_ops.cuh"
#include "gpr_ops15.h"

using namespace gpr;
using namespace gpr::host;
using namespace gpr::multi;

namespace gpr {
namespace host {

int Ops15::boundaries(const double *u, double *ub, const int32_t *nX, int nd,
                        const int32_t *bcs, cudaStream_t st) {
  return Ops<L15>::boundaries(u, ub, nX, nd, bcs, st);
}

long Ops15::weno_scratch(const int32_t *nX, int nd) {
  return Ops<L15>::weno_scratch(nX, nd);
}

int Ops15::weno(double *wh, const double *ub, const int32_t *nX, int nd, double *scratch,
                  cudaStream_t st) {
  return Ops<L15>::weno(wh, ub, nX, nd, scratch, st);
}

int Ops15::predictor(double *qh, const double *wh, double dt, const double *dt_dev,
                       const double *dX, int nd, const int32_t *nX, int stiff,
                       const DevPar &P, const uint8_t *mask, int32_t *status,
                       cudaStream_t st) {
  return Ops<L15>::predictor(qh, wh, dt, dt_dev, dX, nd, nX, stiff, P, mask, status, st);
}

long Ops15::fv_scratch(const int32_t *nX, int nd) {
  return Ops<L15>::fv_scratch(nX, nd);
}

int Ops15::fv(double *u, const double *qh, const int32_t *nX, double dt,
                const double *dt_dev, const double *dX, int nd, int sources, int time_dg,
                const DevPar &P, const uint8_t *mask, double *scratch, cudaStream_t st,
                int flux, int parts) {
  return Ops<L15>::fv(u, qh, nX, dt, dt_dev, dX, nd, sources, time_dg, P, mask, scratch, st, flux,
                      parts);
}

int Ops15::faces(const double *qh, const int32_t *nX, double dt, const double *dX, int nd,
                   int time_dg, const DevPar &P, const uint8_t *mask, double *fb,
                   cudaStream_t st, int flux) {
  return Ops<L15>::faces(qh, nX, dt, dX, nd, time_dg, P, mask, fb, st, flux);
}

int Ops15::timestep(const double *u, long ncell, const double *dX, int nd, double cfl,
                      double t, double tf, int count, const DevPar &P, double *dt_out,
                      double *scratch, cudaStream_t st) {
  return Ops<L15>::timestep(u, ncell, dX, nd, cfl, t, tf, count, P, dt_out, scratch, st);
}

int Ops15::renorm(double *u, long ncell, const DevPar &P, cudaStream_t st) {
  return Ops<L15>::renorm(u, ncell, P, st);
}

void Ops15::contortion(double *u, long ncell, double tol, const DevPar &P0, const DevPar &P1,
                         int *flag, const double *dt_dev, cudaStream_t st) {
  Ops<L15>::contortion(u, ncell, tol, P0, P1, flag, dt_dev, st);
}

int Ops15::pointwise(int what, const double *Q, const double *X, double *out, double *out2,
                       long count, int d, int flux, const DevPar &P, cudaStream_t st) {
  return Ops<L15>::pointwise(what, Q, X, out, out2, count, d, flux, P, st);
}

int Ops15::iterate(double *u, const int32_t *nX, int nd, const double *dX,
                     const int32_t *bcs, const DevPar &P, const uint8_t *mask, double *clk,
                     int nsteps, double *scratch, int32_t *status, cudaStream_t st,
                     int flux, double contorted_tol) {
  return Ops<L15>::iterate(u, nX, nd, dX, bcs, P, mask, clk, nsteps, scratch, status, st, flux, contorted_tol);
}

int Ops15::midstep(double *wh, double dt, const double *dt_dev, const double *dX, int nd,
                     const int32_t *nX, const DevPar &P, const uint8_t *mask, cudaStream_t st) {
  return Ops<L15>::midstep(wh, dt, dt_dev, dX, nd, nX, P, mask, st);
}

int Ops15::split_stepper(double *u, double *ub, const int32_t *nX, int nd, double dt,
                           const double *dt_dev, const double *dX, int half_step, int flux,
                           const DevPar &P, const uint8_t *mask, double *scratch,
                           cudaStream_t st) {
  return Ops<L15>::split_stepper(u, ub, nX, nd, dt, dt_dev, dX, half_step, flux, P, mask, scratch, st);
}

long Ops15::split_scratch(const int32_t *nX, int nd) {
  return Ops<L15>::split_scratch(nX, nd);
}

int Ops15::iterate_split(double *u, const int32_t *nX, int nd, const double *dX,
                           const int32_t *bcs, const DevPar &P, const uint8_t *mask,
                           double *clk, int nsteps, double *scratch, int half_step, int flux,
                           cudaStream_t st, double contorted_tol) {
  return Ops<L15>::iterate_split(u, nX, nd, dX, bcs, P, mask, clk, nsteps, scratch, half_step, flux, st, contorted_tol);
}

long Ops15::iterate_scratch(const int32_t *nX, int nd) {
  return Ops<L15>::iterate_scratch(nX, nd);
}

BatchLayout Ops15::batch_layout(int ninst, const int32_t *nx) {
  return Ops<L15>::batch_layout(ninst, nx);
}

int Ops15::batch_iterate(double *u, double *clk, int ninst, const int32_t *nx, int nsteps,
                           double *scr, int32_t *status, unsigned long long *updates,
                           cudaStream_t st, const BatchShapes &sh) {
  return Ops<L15>::batch_iterate(u, clk, ninst, nx, nsteps, scr, status, updates, st, sh);
}

int Ops15::batch_autotune(double *u, double *clk, int ninst, const int32_t *nx, double *scr,
                            BatchShapes &sh, float *times, int reps, cudaStream_t st) {
  return Ops<L15>::batch_autotune(u, clk, ninst, nx, scr, sh, times, reps, st);
}

int Ops15::ode(double *u, long ncell, double dt, const DevPar &P, cudaStream_t st) {
  return Ops<L15>::ode(u, ncell, dt, P, st);
}

}  // namespace host
}  // namespace gpr

namespace {

constexpr int V15 = 15;
constexpr int kLayers = 10 * NN;  // EXPANSION_FACTOR * N (fill.cpp:258)

Grid make_grid(const int32_t *nX, int nd, const double *dX) {
  Grid g;
  g.nd = nd;
  g.nx = nX[0];
  g.ny = nd == 2 ? nX[1] : 1;
  g.ncell = (long)g.nx * g.ny;
  g.dx = dX[0];
  g.dy = nd == 2 ? dX[1] : 1.0;
  return g;
}

bool grid_ok(const int32_t *nX, int nd) {
  if (!nX || (nd != 1 && nd != 2))
    return false;
  for (int k = 0; k < nd; k++)
    if (nX[k] < 3)
      return false;
  return true;
}

// Sweeps per re-distancing round (a tile's sweeps between halo exchanges):
// a tile converges on a fixed halo within its Manhattan diameter (~2 tile
// widths); the budget only bounds a round.
constexpr int kFmmSweeps = 256;

// Round budget: information crosses at least one tile per round; the
// 800 x 400 shock bubble needs 43 (static circle) to 54 (advected) of its
// 75 tile rows plus columns.  Rounds past convergence return at once but
// still cost a launch, so the budget is that sum plus 16, the last quarter
// of the sum with monotone updates (which guarantees termination).
int fmm_tiles_across(const Grid &g) {
  int tiles = g.nd == 1 ? (g.nx + FMM_T1 - 1) / FMM_T1
                        : (g.nx + FMM_T2 - 1) / FMM_T2 + (g.ny + FMM_T2 - 1) / FMM_T2;
  int sweeps = (g.nx + (g.nd == 2 ? g.ny : 0) + kFmmSweeps - 1) / kFmmSweeps;
  return tiles > sweeps ? tiles : sweeps;
}
int fmm_rounds(const Grid &g) { return fmm_tiles_across(g) + 16; }
int fmm_mono_from(const Grid &g) { return fmm_rounds(g) - fmm_tiles_across(g) / 4 - 4; }

// Scratch of one fill (offsets in doubles, 256-byte aligned pieces).
struct FillLayout {
  long o_d, o_phim, o_dphi, o_star, o_plan, o_fz, o_im0, o_im1, o_lastw, o_pidx, o_dep,
      o_level, o_cnt, o_flags, o_tflag, o_lastg, o_par, o_d2, o_par2, o_list, o_qst, o_gs,
      total;
};

int fmm_tiles(const Grid &g) {
  if (g.nd == 1)
    return (g.nx + FMM_T1 - 1) / FMM_T1;
  return ((g.nx + FMM_T2 - 1) / FMM_T2) * ((g.ny + FMM_T2 - 1) / FMM_T2);
}

FillLayout fill_layout(const Grid &g) {
  auto dbl = [](long bytes) { return (bytes + 7) / 8; };
  long n = g.ncell;
  Carve cv;
  FillLayout L;
  L.o_d = cv.take(n);
  L.o_phim = cv.take(n);
  L.o_dphi = cv.take(n * g.nd);
  L.o_star = cv.take(n * V15);
  L.o_plan = cv.take(dbl(n * (long)sizeof(BPlan)));
  L.o_fz = cv.take(dbl(n));
  L.o_im0 = cv.take(dbl(n * 4));
  L.o_im1 = cv.take(dbl(n * 4));
  L.o_lastw = cv.take(dbl(n * 4));
  L.o_pidx = cv.take(dbl(n * 4));
  L.o_dep = cv.take(dbl(n * 4));
  L.o_level = cv.take(dbl(n * 4));
  L.o_cnt = cv.take(dbl(8 * 4));  // anyfrozen, nplan, maxlevel
  L.o_flags = cv.take(dbl(fmm_rounds(g) * 4L));
  L.o_tflag = cv.take(dbl((long)fmm_rounds(g) * fmm_tiles(g) * 4L));
  L.o_lastg = cv.take(dbl(n * 4));
  L.o_par = cv.take(dbl(n));
  // the 2D global sweeps: second buffers, two work lists, list stamps,
  // counters and the grid barrier
  L.o_d2 = cv.take(n);
  L.o_par2 = cv.take(dbl(n));
  L.o_list = cv.take(dbl(2 * n * 4));
  L.o_qst = cv.take(dbl(n * 4));
  L.o_gs = cv.take(dbl(16 * 4));
  L.total = cv.o;
  return L;
}

// Sweep budget of the 2D global sweeps: the dependency chain of a point is
// at most ~1.5 (nx + ny) sweeps long; from 2 (nx + ny) + 64 sweeps on only
// decreasing updates are taken (termination), and 3 (nx + ny) + 128 ends
// the loop with an error.
int fmm_mono_sweeps(const Grid &g) { return 2 * (g.nx + g.ny) + 64; }
int fmm_max_sweeps(const Grid &g) { return 3 * (g.nx + g.ny) + 128; }

// Blocks of the cooperative k_fmm_global launch: one per SM (the lists
// rarely hold more points than its threads; fewer blocks make the barrier
// cheaper).
int fmm_global_blocks() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && cached[dev] > 0)
    return cached[dev];
  int nsm = 0, per = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fmm_global, 256, 0);
  if (per > 1)
    per = 1;
  const int nb = nsm * (per > 0 ? per : 0);
  if (dev >= 0 && dev < 64)
    cached[dev] = nb;
  return nb;
}

template <class T> T *at(double *scr, long off) { return (T *)(scr + off); }

const int kPlanGrid = 152 * 8;  // grid-stride launches over the plan entries

// Re-distance phi (stride ps) into d; also writes u's level set when u != 0.
int redistance(const double *phi, long ps, double *u, const Grid &g, double *scr,
               const FillLayout &L, int *err, const double *clk, cudaStream_t st,
               int *sweeps = nullptr) {
  double *d = scr + L.o_d;
  uint8_t *fz = at<uint8_t>(scr, L.o_fz);
  int *cnt = at<int>(scr, L.o_cnt), *flags = at<int>(scr, L.o_flags);
  int *tflag = at<int>(scr, L.o_tflag), *lastg = at<int>(scr, L.o_lastg);
  int R = fmm_rounds(g);
  cudaMemsetAsync(cnt, 0, 8 * sizeof(int), st);
  cudaMemsetAsync(flags, 0, R * sizeof(int), st);
  if (g.nd == 1) {
    cudaMemsetAsync(tflag, 0, (size_t)R * fmm_tiles(g) * sizeof(int), st);
    cudaMemsetAsync(lastg, 0xff, g.ncell * sizeof(int), st);
  }
  uint8_t *par = at<uint8_t>(scr, L.o_par);
  k_fmm_init<<<blocks(g.ncell, 256), 256, 0, st>>>(phi, ps, d, fz, par, g, cnt, clk);
  FmmConst K = fmm_const(g.dx, g.nd == 2 ? g.dy : g.dx);
  if (g.nd == 2) {
    FmmGlobal G;
    G.d[0] = d;
    G.d[1] = scr + L.o_d2;
    G.par[0] = par;
    G.par[1] = at<uint8_t>(scr, L.o_par2);
    G.fz = fz;
    G.list[0] = at<int>(scr, L.o_list);
    G.list[1] = G.list[0] + g.ncell;
    G.qst = at<int>(scr, L.o_qst);
    G.cnt = at<int>(scr, L.o_gs);
    G.bar = (unsigned *)(G.cnt + 8);
    G.err = err;
    G.sweeps = sweeps;
    G.mono_from = fmm_mono_sweeps(g);
    G.max_sweeps = fmm_max_sweeps(g);
    const int nb = fmm_global_blocks();
    if (nb <= 0)
      return GPR_E_CUDA;
    cudaMemsetAsync(G.cnt, 0, 16 * sizeof(int), st);
    cudaMemsetAsync(G.qst, 0xff, g.ncell * sizeof(int), st);
    cudaMemcpyAsync(G.d[1], d, g.ncell * sizeof(double), cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(G.par[1], par, g.ncell, cudaMemcpyDeviceToDevice, st);
    k_fmm_seed<<<blocks(g.ncell, 256), 256, 0, st>>>(g, G, clk);
    void *args[] = {(void *)&g, (void *)&K, (void *)&G, (void *)&clk};
    if (cudaLaunchCooperativeKernel((const void *)k_fmm_global, dim3(nb), dim3(256), args, 0,
                                    st) != cudaSuccess)
      return cuda_rc();
    // the sweeps end with both buffers equal (no point changed in the last
    // one); d[0] is d.  flags[0] is zero: the kernel reports its own budget.
    k_fmm_finish<V15><<<blocks(g.ncell, 256), 256, 0, st>>>(d, u, g.ncell, cnt, flags, 0, err,
                                                            clk);
    return cuda_rc();
  } else {
    int nb = (g.nx + FMM_T1 - 1) / FMM_T1;
    for (int r = 0; r < R; r++)
      k_fmm_round<1><<<nb, FmmThreads<1>::value, 0, st>>>(d, fz, par, lastg, g, K, flags, tflag, r,
                                                 kFmmSweeps, r >= fmm_mono_from(g), clk);
  }
  k_fmm_finish<V15><<<blocks(g.ncell, 256), 256, 0, st>>>(d, u, g.ncell, cnt, flags, R - 1, err,
                                                          clk);
  return cuda_rc();
}

// fill_boundary_cells (fill.cpp:200-235) on grid for material mat, given
// its level set phim, normals dphi and interface cells im.
int boundary_fill(double *grid, const double *phim, const double *dphi, const int32_t *im,
                  int mat, const DevPar &P0, const DevPar &P1, double dt, const double *dt_dev,
                  const Grid &g, double *scr, const FillLayout &L, int *err, const double *clk,
                  cudaStream_t st) {
  BPlan *plan = at<BPlan>(scr, L.o_plan);
  int32_t *lastw = at<int32_t>(scr, L.o_lastw), *pidx = at<int32_t>(scr, L.o_pidx);
  int32_t *dep = at<int32_t>(scr, L.o_dep), *level = at<int32_t>(scr, L.o_level);
  int *cnt = at<int>(scr, L.o_cnt);
  double *star = scr + L.o_star;
  cudaMemsetAsync(lastw, 0xff, g.ncell * sizeof(int32_t), st);
  cudaMemsetAsync(cnt + 1, 0, 2 * sizeof(int), st);
  k_plan<V15><<<blocks(g.ncell, 256), 256, 0, st>>>(phim, dphi, im, grid, mat, g, plan,
                                                     cnt + 1, pidx, lastw, err, clk);
  k_plan_deps<<<kPlanGrid, 128, 0, st>>>(plan, cnt + 1, pidx, lastw, dep, clk);
  k_plan_levels<<<kPlanGrid, 128, 0, st>>>(cnt + 1, dep, level, cnt + 2, clk);
  k_star_level0<V15><<<kPlanGrid, 64, 0, st>>>(plan, cnt + 1, dep, level, grid, star, P0, P1,
                                               mat, dt, dt_dev, g.nd, clk);
  k_star_levels<V15><<<1, 64, 0, st>>>(plan, cnt + 1, dep, level, cnt + 2, grid, star, P0,
                                       P1, mat, dt, dt_dev, g.nd, clk);
  k_scatter<V15><<<kPlanGrid, 128, 0, st>>>(plan, cnt + 1, lastw, star, grid, clk);
  return cuda_rc();
}

// fill_neighbor_cells (fill.cpp:255-328); im is updated in place (the
// second buffer is scratch).
int neighbor_fill(double *grid, int32_t *im, int32_t *im2, const double *dphi, const Grid &g,
                  int *err, const double *clk, cudaStream_t st) {
  int32_t *a = im, *b = im2;
  for (int N0 = 1; N0 < kLayers; N0++) {
    k_layer<V15><<<blocks(g.ncell, 256), 256, 0, st>>>(grid, a, b, dphi, g, N0, err, clk);
    int32_t *t = a;
    a = b;
    b = t;
  }
  if (a != im)
    cudaMemcpyAsync(im, a, g.ncell * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  return cuda_rc();
}

// fill_ghost_cells (fill.cpp:330-370) for two materials.
int fill(double *grids, uint8_t *masks, double *u, const Grid &g, double dt,
         const double *dt_dev, const DevPar P[2], double *scr, const FillLayout &L, int *err,
         const double *clk, cudaStream_t st) {
  int rc = redistance(u + V15 - 1, V15, u, g, scr, L, err, clk, st);
  if (rc)
    return rc;
  double *d = scr + L.o_d, *phim = scr + L.o_phim, *dphi = scr + L.o_dphi;
  int32_t *im = at<int32_t>(scr, L.o_im0), *im2 = at<int32_t>(scr, L.o_im1);
  for (int mat = 0; mat < 2; mat++) {
    double *grid = grids + (long)mat * g.ncell * V15;
    uint8_t *mask = masks + (long)mat * g.ncell;
    if (P[mat].EOS <= -1) {
      cudaMemsetAsync(mask, 0, g.ncell, st);
      continue;
    }
    cudaMemcpyAsync(grid, u, g.ncell * V15 * sizeof(double), cudaMemcpyDeviceToDevice, st);
    k_mat_phi<<<blocks(g.ncell, 256), 256, 0, st>>>(d, mat == 0 ? 1 : -1, phim, g.ncell, clk);
    k_finite_difference<<<blocks(g.ncell, 256), 256, 0, st>>>(phim, dphi, g, clk);
    k_interface_cells<<<blocks(g.ncell, 256), 256, 0, st>>>(phim, im, g, clk);
    if ((rc = boundary_fill(grid, phim, dphi, im, mat, P[0], P[1], dt, dt_dev, g, scr, L, err,
                            clk, st)))
      return rc;
    if ((rc = neighbor_fill(grid, im, im2, dphi, g, err, clk, st)))
      return rc;
    k_mat_mask<<<blocks(g.ncell, 256), 256, 0, st>>>(phim, im, mask, g.ncell, clk);
  }
  return cuda_rc();
}

// Scratch of the two-material time loop.
struct MultiLayout {
  FillLayout f;
  long o_fill, o_grids, o_masks, o_maskb, o_ub, o_wh, o_qh, o_tmp, o_mx, o_flag, o_pst, total;
};

MultiLayout multi_layout(const int32_t *nX, int nd, const Grid &g) {
  auto dbl = [](long bytes) { return (bytes + 7) / 8; };
  MultiLayout M;
  M.f = fill_layout(g);
  long ncb = nd == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
  long nub = nd == 1 ? nX[0] + 2 * NN : (long)(nX[0] + 2 * NN) * (nX[1] + 2 * NN);
  long ns = nd == 1 ? NN : NN * NN;
  long w = Ops<L15>::weno_scratch(nX, nd), f = Ops<L15>::fv_scratch(nX, nd);
  Carve cv;
  M.o_fill = cv.take(M.f.total);
  M.o_grids = cv.take(2 * g.ncell * V15);
  M.o_masks = cv.take(dbl(2 * g.ncell));
  M.o_maskb = cv.take(dbl(ncb));
  M.o_ub = cv.take(nub * V15);
  M.o_wh = cv.take(ncb * ns * V15);
  M.o_qh = cv.take(ncb * NN * ns * V15);
  M.o_tmp = cv.take(w > f ? w : f);
  M.o_mx = cv.take(1);
  M.o_flag = cv.take(1);
  M.o_pst = cv.take(dbl(ncb * 4));
  M.total = cv.o;
  return M;
}

int check_pars(const gpr_par *pars, int nmat, DevPar P[2]) {
  if (!pars || nmat != 2)
    return GPR_E_ARG;
  for (int m = 0; m < 2; m++)
    P[m] = make_devpar(pars[m]);
  if (P[0].EOS <= -1 && P[1].EOS <= -1)
    return GPR_E_ARG;
  return GPR_OK;
}

}  // namespace

extern "C" {

long gpr_distance_scratch_doubles(const int32_t *nX, int ndim) {
  if (!grid_ok(nX, ndim))
    return GPR_E_ARG;
  double dX[2] = {1.0, 1.0};
  return fill_layout(make_grid(nX, ndim, dX)).total;
}

int gpr_distance(const double *phi, double *dist, const int32_t *nX, int ndim,
                 const double *dX, double *scratch, int32_t *status, void *stream) {
  if (!phi || !dist || !dX || !scratch || !status || !grid_ok(nX, ndim))
    return GPR_E_ARG;
  Grid g = make_grid(nX, ndim, dX);
  FillLayout L = fill_layout(g);
  cudaStream_t st = S(stream);
  int rc = redistance(phi, 1, nullptr, g, scratch, L, status, nullptr, st, status + 3);
  if (rc)
    return rc;
  cudaMemcpyAsync(dist, scratch + L.o_d, g.ncell * sizeof(double), cudaMemcpyDeviceToDevice,
                  st);
  return cuda_rc();
}

int gpr_finite_difference(const double *phi, double *dphi, const int32_t *nX, int ndim,
                          const double *dX, void *stream) {
  if (!phi || !dphi || !dX || !grid_ok(nX, ndim))
    return GPR_E_ARG;
  Grid g = make_grid(nX, ndim, dX);
  k_finite_difference<<<blocks(g.ncell, 256), 256, 0, S(stream)>>>(phi, dphi, g, nullptr);
  return cuda_rc();
}

int gpr_find_interface_cells(const double *phi, int32_t *intMask, const int32_t *nX, int ndim,
                             void *stream) {
  if (!phi || !intMask || !grid_ok(nX, ndim))
    return GPR_E_ARG;
  double dX[2] = {1.0, 1.0};
  Grid g = make_grid(nX, ndim, dX);
  k_interface_cells<<<blocks(g.ncell, 256), 256, 0, S(stream)>>>(phi, intMask, g, nullptr);
  return cuda_rc();
}

int gpr_left_star_state(const double *QL, const double *QR, const double *n, double *out,
                        int64_t count, int ndim, double dt, const gpr_par *parL,
                        const gpr_par *parR, int nvar, void *stream) {
  if (!QL || !QR || !n || !out || !parL || !parR || count < 0 || (ndim != 1 && ndim != 2))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  if (count == 0)
    return GPR_OK;
  k_star_pointwise<V15><<<blocks(count, 64), 64, 0, S(stream)>>>(
      QL, QR, n, out, count, ndim, dt, make_devpar(*parL), make_devpar(*parR));
  return cuda_rc();
}

long gpr_fill_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!grid_ok(nX, ndim))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  double dX[2] = {1.0, 1.0};
  return fill_layout(make_grid(nX, ndim, dX)).total;
}

int gpr_fill_boundary_cells(double *grid, const int32_t *intMask, int mat, const double *phi,
                            const double *dphi, const double *dX, const gpr_par *pars,
                            int nmat, double dt, const int32_t *nX, int ndim, double *scratch,
                            int32_t *status, int nvar, void *stream) {
  if (!grid || !intMask || !phi || !dphi || !dX || !scratch || !status || mat < 0 || mat > 1 ||
      !grid_ok(nX, ndim))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  DevPar P[2];
  if (int rc = check_pars(pars, nmat, P))
    return rc;
  Grid g = make_grid(nX, ndim, dX);
  return boundary_fill(grid, phi, dphi, intMask, mat, P[0], P[1], dt, nullptr, g, scratch,
                       fill_layout(g), status, nullptr, S(stream));
}

int gpr_fill_neighbor_cells(double *grid, int32_t *intMask, const double *dphi,
                            const double *dX, const int32_t *nX, int ndim, double *scratch,
                            int32_t *status, int nvar, void *stream) {
  if (!grid || !intMask || !dphi || !dX || !scratch || !status || !grid_ok(nX, ndim))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  Grid g = make_grid(nX, ndim, dX);
  FillLayout L = fill_layout(g);
  return neighbor_fill(grid, intMask, at<int32_t>(scratch, L.o_im1), dphi, g, status, nullptr,
                       S(stream));
}

int gpr_fill_ghost_cells(double *grids, uint8_t *masks, double *u, const int32_t *nX, int ndim,
                         const double *dX, double dt, const gpr_par *pars, int nmat,
                         double *scratch, int32_t *status, int nvar, void *stream) {
  if (!grids || !masks || !u || !dX || !scratch || !status || !grid_ok(nX, ndim))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  DevPar P[2];
  if (int rc = check_pars(pars, nmat, P))
    return rc;
  Grid g = make_grid(nX, ndim, dX);
  return fill(grids, masks, u, g, dt, nullptr, P, scratch, fill_layout(g), status, nullptr,
              S(stream));
}

int gpr_make_u(double *u, const double *grids, const uint8_t *masks, int64_t ncell,
               const gpr_par *pars, int nmat, int nvar, void *stream) {
  if (!u || !grids || !masks || ncell < 1)
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  DevPar P[2];
  if (int rc = check_pars(pars, nmat, P))
    return rc;
  k_make_u<V15><<<blocks(ncell, 256), 256, 0, S(stream)>>>(u, grids, masks, ncell, 2, P[0].EOS,
                                                           P[1].EOS, nullptr);
  return cuda_rc();
}

int gpr_renorm_multi(double *u, int64_t ncell, const gpr_par *pars, int nmat, int nvar,
                     void *stream) {
  if (!u || ncell < 1)
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  DevPar P[2];
  if (int rc = check_pars(pars, nmat, P))
    return rc;
  k_renorm_multi<V15><<<blocks(ncell, 256), 256, 0, S(stream)>>>(u, ncell, P[0].rho0,
                                                                 P[1].rho0, P[0].EOS, P[1].EOS,
                                                                 nullptr);
  return cuda_rc();
}

int gpr_timestep_multi(const double *grids, const uint8_t *masks, int64_t ncell,
                       const double *dX, int ndim, double cfl, double t, double tf, int count,
                       const gpr_par *pars, int nmat, double *dt_out, double *scratch,
                       int nvar, void *stream) {
  if (!grids || !masks || !dX || !dt_out || !scratch || ncell < 1 || (ndim != 1 && ndim != 2))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  DevPar P[2];
  if (int rc = check_pars(pars, nmat, P))
    return rc;
  cudaStream_t st = S(stream);
  unsigned long long *mx = (unsigned long long *)scratch;
  cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st);
  for (int m = 0; m < 2; m++)
    if (P[m].EOS > -1)
      k_cfl_max_masked<L15><<<blocks(ncell, 256), 256, 0, st>>>(
          grids + (long)m * ncell * V15, masks + (long)m * ncell, ncell, ndim, dX[0],
          ndim == 2 ? dX[1] : 1.0, mx, P[m], nullptr);
  k_cfl_finalize<<<1, 1, 0, st>>>(mx, cfl, t, tf, count, dt_out);
  return cuda_rc();
}

long gpr_iterate_multi_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!grid_ok(nX, ndim))
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  double dX[2] = {1.0, 1.0};
  return multi_layout(nX, ndim, make_grid(nX, ndim, dX)).total;
}

// The two-material loop of solvers/iterator.cpp:85-170 (LSET > 0): fill ->
// CFL over the masked cells of both grids -> per material boundaries,
// extended mask and the masked step (the ADER scheme, or the split scheme
// when split != 0, iterator.cpp:123-129) -> make_u -> renorm -> contortion
// check and reset (solvers/utils.cpp:44-85) -> clock.  The clock
// {t, dt, tf, cfl, count} lives on the device; the fill of a step uses the
// previous step's dt, as the reference does.
static int iterate_multi(double *u, const int32_t *nX, int ndim, const double *dX,
                         const int32_t *bcs, int split, int half_step, int stiff, int flux,
                         const gpr_par *pars, int nmat, double *clock, int nsteps,
                         double *scratch, int32_t *status, double contorted_tol, int nvar,
                         void *stream) {
  if (!u || !dX || !bcs || !clock || !scratch || !status || nsteps < 0 || !grid_ok(nX, ndim))
    return GPR_E_ARG;
  for (int i = 0; i < 2 * ndim; i++)
    if (bcs[i] < 0 || bcs[i] > 5)
      return GPR_E_ARG;
  if (flux != GPR_FLUX_RUSANOV && flux != GPR_FLUX_ROE && flux != GPR_FLUX_OSHER)
    return GPR_E_ARG;
  if (nvar != V15)
    return GPR_E_UNSUPPORTED;
  DevPar P[2];
  if (int rc = check_pars(pars, nmat, P))
    return rc;
  Grid g = make_grid(nX, ndim, dX);
  MultiLayout M = multi_layout(nX, ndim, g);
  cudaStream_t st = S(stream);
  double *fs = scratch + M.o_fill, *grids = scratch + M.o_grids;
  uint8_t *masks = at<uint8_t>(scratch, M.o_masks), *maskb = at<uint8_t>(scratch, M.o_maskb);
  double *ub = scratch + M.o_ub, *wh = scratch + M.o_wh, *qh = scratch + M.o_qh;
  double *tmp = scratch + M.o_tmp;
  unsigned long long *mx = (unsigned long long *)(scratch + M.o_mx);
  int32_t *pst = at<int32_t>(scratch, M.o_pst);
  double *dt_dev = clock + 1;
  for (int s = 0; s < nsteps; s++) {
    int rc = fill(grids, masks, u, g, 0.0, dt_dev, P, fs, M.f, status, clock, st);
    if (rc)
      return rc;
    cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st);
    for (int m = 0; m < 2; m++)
      if (P[m].EOS > -1)
        k_cfl_max_masked<L15><<<blocks(g.ncell, 256), 256, 0, st>>>(
            grids + (long)m * g.ncell * V15, masks + (long)m * g.ncell, g.ncell, ndim, g.dx,
            g.dy, mx, P[m], clock);
    k_clock_finalize<<<1, 1, 0, st>>>(mx, clock);
    for (int m = 0; m < 2; m++) {
      if (P[m].EOS <= -1)
        continue;
      double *grid = grids + (long)m * g.ncell * V15;
      if ((rc = Ops<L15>::boundaries(grid, ub, nX, ndim, bcs, st)))
        return rc;
      if ((rc = gpr_extend_mask(masks + (long)m * g.ncell, maskb, nX, ndim, st)))
        return rc;
      if (split) {
        // split_stepper's scratch (wh, then the WENO / FV temporary) spans
        // the wh, qh and tmp regions, which lie back to back
        if ((rc = Ops<L15>::split_stepper(grid, ub, nX, ndim, 0.0, dt_dev, dX, half_step, flux,
                                          P[m], maskb, wh, st)))
          return rc;
        continue;
      }
      if ((rc = Ops<L15>::weno(wh, ub, nX, ndim, tmp, st)))
        return rc;
      if ((rc = Ops<L15>::predictor(qh, wh, 0.0, dt_dev, dX, ndim, nX, stiff, P[m], maskb, pst,
                                    st, tmp)))
        return rc;
      if ((rc = Ops<L15>::fv(grid, qh, nX, 0.0, dt_dev, dX, ndim, 1, 1, P[m], maskb, tmp, st,
                             flux)))
        return rc;
    }
    k_make_u<V15><<<blocks(g.ncell, 256), 256, 0, st>>>(u, grids, masks, g.ncell, 2, P[0].EOS,
                                                        P[1].EOS, dt_dev);
    k_renorm_multi<V15><<<blocks(g.ncell, 256), 256, 0, st>>>(
        u, g.ncell, P[0].rho0, P[1].rho0, P[0].EOS, P[1].EOS, dt_dev);
    Ops<L15>::contortion(u, g.ncell, contorted_tol, P[0], P[1], at<int>(scratch, M.o_flag),
                         dt_dev, st);
    k_clock_advance<<<1, 1, 0, st>>>(clock);
  }
  return cuda_rc();
}

int gpr_iterate_multi(double *u, const int32_t *nX, int ndim, const double *dX,
                      const int32_t *bcs, int flux, const gpr_par *pars, int nmat,
                      double *clock, int nsteps, double *scratch, int32_t *status,
                      double contorted_tol, int nvar, void *stream) {
  return iterate_multi(u, nX, ndim, dX, bcs, 0, 0, 0, flux, pars, nmat, clock, nsteps,
                       scratch, status, contorted_tol, nvar, stream);
}

int gpr_iterate_multi_scheme(double *u, const int32_t *nX, int ndim, const double *dX,
                             const int32_t *bcs, int split, int half_step, int stiff, int flux,
                             const gpr_par *pars, int nmat, double *clock, int nsteps,
                             double *scratch, int32_t *status, double contorted_tol, int nvar,
                             void *stream) {
  return iterate_multi(u, nX, ndim, dX, bcs, split, half_step, stiff, flux, pars, nmat, clock,
                       nsteps, scratch, status, contorted_tol, nvar, stream);
}

}  // extern "C"
