// gpr_host.cuh - host-side helpers shared by the C ABI translation units:
// constants, launch sizing, the packed layout of the batched form and the
// persistent launch of the stiff-source Newton pass.
#pragma once

#include <stdio.h>

#include "gpr_kernels.cuh"

namespace gpr {
namespace host {

inline const Consts &consts() {
  static Consts c = make_consts();
  return c;
}

inline cudaStream_t S(void *s) { return (cudaStream_t)s; }

inline int blocks(long n, int bs) { return (int)((n + bs - 1) / bs); }

// SMs of the current device, read once per device.
inline int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64)
    return 152;
  if (!cache[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = n > 0 ? n : 152;
  }
  return cache[dev];
}

// Threads per block for n threads of a kernel written for bs (a power of
// two): halved, down to one warp, while the grid would hold fewer than two
// blocks per SM.  On GB300 a warp issues one FP64 instruction per ~63
// cycles whatever its active lanes, and an SM one per ~19 cycles over all
// its warps, so the few warps of a small grid (the 200-cell tube) finish
// their FP64 chains sooner on separate SMs than four or eight to an SM.
// For kernels whose threads are independent, or whose block reduction is a
// max, the result is the same at any block size.
inline int spread(long n, int bs) {
  const long want = 2L * sm_count();
  while (bs > 32 && (n + bs - 1) / bs < want)
    bs >>= 1;
  return bs;
}

// grid and block of a launch of n threads shaped by spread()
#define GPR_SPREAD(n, bs) blocks((n), spread((n), (bs))), spread((n), (bs))

inline int cuda_rc() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "gpr_gb300: CUDA error %s\n", cudaGetErrorString(e));
    return GPR_E_CUDA;
  }
  return GPR_OK;
}

// 256-byte aligned pieces of a scratch buffer (offsets in doubles)
struct Carve {
  long o = 0;
  long take(long ndoubles) {
    long at = o;
    o += (ndoubles + 31) & ~31L;
    return at;
  }
};

// Launch shapes of the batched step: threads per block of each stage (so
// cells per block = threads / lanes per cell) and the lane layout of the
// face pass.  The defaults are the single-grid kernels' shapes;
// Ops::batch_autotune measures the candidates on a batch and picks the
// fastest of each.
struct BatchShapes {
  int weno = 256;       // k_b_weno: one thread per (cell, variable)
  int first = 128;      // k_predictor_first: 2 lanes per predictor cell
  int picard = 128;     // k_predictor_picard: 4 lanes per predictor cell
  int faces_split = 0;  // 0: k_faces1d (2 lanes per face), 1: k_faces1d_split (4)
  int faces = 128;      // threads per block of the face kernel
  int cells = 128;      // k_cells: 4 lanes per cell
};

// Packed sizes and scratch offsets (in doubles) of the batched form.
struct BatchLayout {
  long nu = 0, nub = 0, nb = 0, nf = 0;
  long o_par, o_iu, o_iub, o_ib, o_if, o_nx, o_ou, o_oub, o_ob, o_of, o_bc, o_idx, o_mx;
  long o_ub, o_wh, o_qh, o_fb, o_rlist, o_rn, o_rit, o_rdmin, total;
};

inline BatchLayout batch_layout_v(int ninst, const int32_t *nx, int V) {
  BatchLayout b;
  for (int k = 0; k < ninst; k++) {
    b.nu += nx[k];
    b.nub += nx[k] + 2 * NN;
    b.nb += nx[k] + 2;
    b.nf += nx[k] + 1;
  }
  auto dbl = [](long bytes) { return (bytes + 7) / 8; };
  Carve cv;
  b.o_par = cv.take(dbl((long)ninst * sizeof(DevPar)));
  b.o_iu = cv.take(dbl(b.nu * 4));
  b.o_iub = cv.take(dbl(b.nub * 4));
  b.o_ib = cv.take(dbl(b.nb * 4));
  b.o_if = cv.take(dbl(b.nf * 4));
  b.o_nx = cv.take(dbl(ninst * 4L));
  b.o_ou = cv.take(dbl(ninst * 4L));
  b.o_oub = cv.take(dbl(ninst * 4L));
  b.o_ob = cv.take(dbl(ninst * 4L));
  b.o_of = cv.take(dbl(ninst * 4L));
  b.o_bc = cv.take(dbl(ninst * 8L));
  b.o_idx = cv.take(ninst);
  b.o_mx = cv.take(ninst);
  b.o_ub = cv.take(b.nub * V);
  b.o_wh = cv.take(b.nb * NN * V);
  b.o_qh = cv.take(b.nb * NN * NN * V);
  b.o_fb = cv.take(b.nf * 2 * V);
  b.o_rlist = cv.take(dbl(b.nb * 4));
  b.o_rn = cv.take(1);
  b.o_rit = cv.take(dbl(b.nb * 4));
  b.o_rdmin = cv.take(b.nb);
  b.total = cv.o;
  return b;
}

inline Batch batch_view_of(double *scr, int ninst, const BatchLayout &b, double *clk) {
  Batch B;
  B.P = (const DevPar *)(scr + b.o_par);
  B.inst_u = (const int32_t *)(scr + b.o_iu);
  B.inst_ub = (const int32_t *)(scr + b.o_iub);
  B.inst_b = (const int32_t *)(scr + b.o_ib);
  B.inst_f = (const int32_t *)(scr + b.o_if);
  B.nx = (const int32_t *)(scr + b.o_nx);
  B.off_u = (const int32_t *)(scr + b.o_ou);
  B.off_ub = (const int32_t *)(scr + b.o_oub);
  B.off_b = (const int32_t *)(scr + b.o_ob);
  B.off_f = (const int32_t *)(scr + b.o_of);
  B.bc = (const int32_t *)(scr + b.o_bc);
  B.idx = scr + b.o_idx;
  B.clk = clk;
  B.ninst = ninst;
  return B;
}

// Stiff-source Newton pass over the cells the Picard pass flagged: a
// persistent grid sized by occupancy (the kernel strides over the cells).
template <class L, int ND, bool BATCH>
int launch_stiff(double *qh, const double *wh, long ncb, const uint8_t *mask, int32_t *status,
                 double dt, const double *dt_dev, double idx, double idy, const DevPar &P,
                 const Consts &C, cudaStream_t st, const Batch &B) {
  constexpr int NP = ND == 1 ? NN * NN : NN * NN * NN;
  constexpr int BS = 64;
  size_t smem = (size_t)(BS / NP) * StiffSmem<L, ND>::per_cell * sizeof(float);
  // per device and cheap: set on every call
  cudaFuncSetAttribute(k_predictor_stiff<L, ND, BATCH>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int dev = 0, nsm = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_predictor_stiff<L, ND, BATCH>, BS,
                                                smem);
  long need = (ncb * NP + BS - 1) / BS;
  long grid = (long)nsm * (per_sm > 0 ? per_sm : 1);
  if (grid > need)
    grid = need;
  k_predictor_stiff<L, ND, BATCH><<<(int)grid, BS, smem, st>>>(qh, wh, ncb, mask, status, dt,
                                                                dt_dev, idx, idy, P, C, B);
  return cuda_rc();
}

}  // namespace host
}  // namespace gpr
