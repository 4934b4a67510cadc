// gpr_capi.cu - C ABI of the GB300 GPR ADER-WENO step (include/gpr_gb300.h).
//
// Host launchers: argument checks, variant dispatch on the number of
// variables (V = 17: viscous + heat conduction; V = 14: viscous; V = 15:
// viscous with one level set, whose launchers live in gpr_multi.cu), grid
// sizing and the stage sequence of one ADER step.  All device work is
// stream-ordered on the caller's stream; nothing here synchronises.
#include <mutex>
#include <stdio.h>

#include "gpr_ops.cuh"
#include "gpr_ops15.h"

using namespace gpr;
using namespace gpr::host;

namespace {

// extend_mask (etc/grid.cpp:176-230): one thread per predictor cell.
__global__ void k_extend_mask(const uint8_t *__restrict__ mask, uint8_t *__restrict__ maskb,
                              int nx, int ny, int nd) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (nd == 1) {
    if (idx >= nx + 2)
      return;
    int i = (int)idx - 1;
    auto m = [&](int k) { return mask[k] != 0; };
    int ii = i < 0 ? 0 : (i > nx - 1 ? nx - 1 : i);  // maskb(0)=maskb(1), maskb(nx+1)=maskb(nx)
    bool v = m(ii) || (ii > 0 && m(ii - 1)) || (ii < nx - 1 && m(ii + 1));
    maskb[idx] = v;
    return;
  }
  long nb = (long)(nx + 2) * (ny + 2);
  if (idx >= nb)
    return;
  int bi = idx / (ny + 2), bj = idx % (ny + 2);
  int i = bi - 1, j = bj - 1;
  bool v;
  bool ei = i < 0 || i > nx - 1, ej = j < 0 || j > ny - 1;
  if (ei && ej)
    v = false;  // corners
  else if (ei)
    v = mask[(long)(i < 0 ? 0 : nx - 1) * ny + j] != 0;
  else if (ej)
    v = mask[(long)i * ny + (j < 0 ? 0 : ny - 1)] != 0;
  else {
    long ind = (long)i * ny + j;
    v = mask[ind] || (i > 0 && mask[ind - ny]) || (i < nx - 1 && mask[ind + ny]) ||
        (j > 0 && mask[ind - 1]) || (j < ny - 1 && mask[ind + 1]);
  }
  maskb[idx] = v;
}


bool check_grid(const int32_t *nX, int nd) {
  if (!nX || (nd != 1 && nd != 2))
    return false;
  for (int d = 0; d < nd; d++)
    if (nX[d] < 1)
      return false;
  return true;
}

// Rusanov, Roe and Osher in 1D and 2D.
int check_flux(int flux, int nd) {
  (void)nd;
  if (flux < GPR_FLUX_RUSANOV || flux > GPR_FLUX_OSHER)
    return GPR_E_ARG;
  return GPR_OK;
}

#define DISPATCH(nvar, CALL)                                                                 \
  switch (nvar) {                                                                            \
  case 17: {                                                                                 \
    using O = Ops<L17>;                                                                      \
    return CALL;                                                                             \
  }                                                                                          \
  case 14: {                                                                                 \
    using O = Ops<L14>;                                                                      \
    return CALL;                                                                             \
  }                                                                                          \
  case 15: {                                                                                 \
    using O = Ops15;                                                                         \
    return CALL;                                                                             \
  }                                                                                          \
  default:                                                                                   \
    return GPR_E_UNSUPPORTED;                                                                \
  }

}  // namespace

extern "C" {

int gpr_version(void) { return 100; }

int gpr_scheme_constants(double *out, int n) {
  constexpr int COUNT = 4 * NN + 2 * NN * NN;  // nodes, weights, end values; 2 N x N
  if (!out || n < COUNT)
    return GPR_E_ARG;
  const Consts &C = consts();  // host values (make_consts), no device call
  int k = 0;
  for (int i = 0; i < NN; i++)
    out[k++] = C.nodes[i];
  for (int i = 0; i < NN; i++)
    out[k++] = C.w[i];
  for (int e = 0; e < 2; e++)
    for (int j = 0; j < NN; j++)
      out[k++] = C.endv[e][j];
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      out[k++] = C.derv[i][j];
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      out[k++] = C.sig[i][j];
  return k;
}

int gpr_supported_nvars(int32_t *out, int cap) {
  static const int32_t vs[] = {17, 14, 15};
  int n = 0;
  for (int i = 0; i < 3 && i < cap; i++)
    out[n++] = vs[i];
  return 3;
}

int gpr_extend_mask(const uint8_t *mask, uint8_t *maskb, const int32_t *nX, int ndim,
                    void *stream) {
  if (!mask || !maskb || !check_grid(nX, ndim))
    return GPR_E_ARG;
  int nx = nX[0], ny = ndim == 2 ? nX[1] : 1;
  long nb = ndim == 1 ? nx + 2 : (long)(nx + 2) * (ny + 2);
  k_extend_mask<<<blocks(nb, 256), 256, 0, S(stream)>>>(mask, maskb, nx, ny, ndim);
  return cuda_rc();
}

int gpr_flux(const double *Q, double *out, int64_t count, int d, const gpr_par *par, int nvar,
             void *stream) {
  if (!Q || !out || count < 0 || d < 0 || d > 2 || !par)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(0, Q, nullptr, out, nullptr, count, d, 0, P, S(stream)))
}

int gpr_source(const double *Q, double *out, int64_t count, const gpr_par *par, int nvar,
               void *stream) {
  if (!Q || !out || count < 0 || !par)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(1, Q, nullptr, out, nullptr, count, 0, 0, P, S(stream)))
}

int gpr_Bdot(const double *Q, const double *x, double *out, int64_t count, int d,
             const gpr_par *par, int nvar, void *stream) {
  if (!Q || !x || !out || count < 0 || d < 0 || d > 2 || !par)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(2, Q, x, out, nullptr, count, d, 0, P, S(stream)))
}

int gpr_max_abs_eigs(const double *Q, double *out, int64_t count, int d, const gpr_par *par,
                     int nvar, void *stream) {
  if (!Q || !out || count < 0 || d < 0 || d > 2 || !par)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(3, Q, nullptr, out, nullptr, count, d, 0, P, S(stream)))
}

int gpr_system_matrix(const double *Q, double *out, int64_t count, int d, const gpr_par *par,
                      int nvar, void *stream) {
  if (!Q || !out || count < 0 || d < 0 || d > 2 || !par)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(5, Q, nullptr, out, nullptr, count, d, 0, P, S(stream)))
}

int gpr_thermo_acoustic_tensor(const double *Q, double *out, int64_t count, int d,
                               const gpr_par *par, int nvar, void *stream) {
  if (!Q || !out || count < 0 || d < 0 || d > 2 || !par)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(6, Q, nullptr, out, nullptr, count, d, 0, P, S(stream)))
}

int gpr_interface_terms(const double *qL, const double *qR, double *out, double *bout,
                        int64_t count, int d, int flux, const gpr_par *par, int nvar,
                        void *stream) {
  if (!qL || !qR || !out || !bout || count < 0 || d < 0 || d > 2 || !par)
    return GPR_E_ARG;
  if (flux < GPR_FLUX_RUSANOV || flux > GPR_FLUX_OSHER)
    return GPR_E_ARG;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::pointwise(4, qL, qR, out, bout, count, d, flux, P, S(stream)))
}

int gpr_boundaries(const double *u, double *ub, const int32_t *nX, int ndim,
                   const int32_t *bcs, int nvar, void *stream) {
  if (!u || !ub || !bcs || !check_grid(nX, ndim))
    return GPR_E_ARG;
  for (int i = 0; i < 2 * ndim; i++)
    if (bcs[i] < 0 || bcs[i] > 5)
      return GPR_E_ARG;
  DISPATCH(nvar, O::boundaries(u, ub, nX, ndim, bcs, S(stream)))
}

long gpr_weno_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!check_grid(nX, ndim))
    return GPR_E_ARG;
  DISPATCH(nvar, O::weno_scratch(nX, ndim))
}

int gpr_weno_launcher(double *wh, const double *ub, const int32_t *nX, int ndim,
                      double *scratch, int nvar, void *stream) {
  if (!wh || !ub || !check_grid(nX, ndim))
    return GPR_E_ARG;
  DISPATCH(nvar, O::weno(wh, ub, nX, ndim, scratch, S(stream)))
}

int gpr_predictor(double *qh, const double *wh, double dt, const double *dX, int ndim,
                  const int32_t *nX, int stiff, const gpr_par *par, const uint8_t *mask,
                  int32_t *status, int nvar, void *stream) {
  if (!qh || !wh || !dX || !par || !check_grid(nX, ndim))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::predictor(qh, wh, dt, nullptr, dX, ndim, nX, stiff, P, mask, status,
                              S(stream)))
}

long gpr_fv_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!check_grid(nX, ndim))
    return GPR_E_ARG;
  DISPATCH(nvar, O::fv_scratch(nX, ndim))
}

int gpr_fv_launcher(double *u, const double *qh, const int32_t *nX, double dt,
                    const double *dX, int ndim, int sources, int time_dg, int flux,
                    const gpr_par *par, const uint8_t *mask, double *scratch, int nvar,
                    void *stream) {
  if (!u || !qh || !dX || !par || !check_grid(nX, ndim) ||
      (!scratch && flux != GPR_FLUX_RUSANOV))
    return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::fv(u, qh, nX, dt, nullptr, dX, ndim, sources, time_dg, P, mask, scratch,
                       S(stream), flux))
}

int gpr_fv_centers(double *u, const double *qh, const int32_t *nX, double dt,
                   const double *dX, int ndim, int sources, int time_dg, const gpr_par *par,
                   const uint8_t *mask, int nvar, void *stream) {
  if (!u || !qh || !dX || !par || !check_grid(nX, ndim))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::fv(u, qh, nX, dt, nullptr, dX, ndim, sources, time_dg, P, mask, nullptr,
                       S(stream), GPR_FLUX_RUSANOV, 1))
}

int gpr_fv_interfs(double *u, const double *qh, const int32_t *nX, double dt,
                   const double *dX, int ndim, int time_dg, int flux, const gpr_par *par,
                   const uint8_t *mask, double *scratch, int nvar, void *stream) {
  if (!u || !qh || !dX || !par || !check_grid(nX, ndim) ||
      (!scratch && flux != GPR_FLUX_RUSANOV))
    return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::fv(u, qh, nX, dt, nullptr, dX, ndim, 0, time_dg, P, mask, scratch,
                       S(stream), flux, 2))
}

int gpr_fv_face_fluxes(const double *qh, const int32_t *nX, double dt, const double *dX,
                       int ndim, int time_dg, int flux, const gpr_par *par,
                       const uint8_t *mask, double *fb, int nvar, void *stream) {
  if (!qh || !dX || !par || !fb || !check_grid(nX, ndim))
    return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::faces(qh, nX, dt, dX, ndim, time_dg, P, mask, fb, S(stream), flux))
}

int gpr_timestep_scratch_doubles(int64_t ncell) {
  (void)ncell;
  return 1;
}

int gpr_timestep(const double *u, int64_t ncell, const double *dX, int ndim, double cfl,
                 double t, double tf, int count, const gpr_par *par, double *dt_out,
                 double *scratch, int nvar, void *stream) {
  if (!u || ncell < 1 || !dX || (ndim != 1 && ndim != 2) || !par || !dt_out || !scratch)
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::timestep(u, ncell, dX, ndim, cfl, t, tf, count, P, dt_out, scratch,
                             S(stream)))
}

int gpr_renorm_distortion(double *u, int64_t ncell, const gpr_par *par, int nvar,
                          void *stream) {
  if (!u || ncell < 0 || !par)
    return GPR_E_ARG;
  if (ncell == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::renorm(u, ncell, P, S(stream)))
}

int gpr_ode_launcher(double *u, int64_t ncell, double dt, const gpr_par *par, int nvar,
                     void *stream) {
  if (!u || ncell < 0 || !par)
    return GPR_E_ARG;
  if (ncell == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::ode(u, ncell, dt, P, S(stream)))
}

long gpr_ader_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!check_grid(nX, ndim))
    return GPR_E_ARG;
  long ncb = ndim == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
  long ns = ndim == 1 ? NN : NN * NN;
  long wh = ncb * ns * nvar, qh = ncb * NN * ns * nvar;
  long w = gpr_weno_scratch_doubles(nX, ndim, nvar);
  long f = gpr_fv_scratch_doubles(nX, ndim, nvar);
  if (w < 0 || f < 0)
    return GPR_E_UNSUPPORTED;
  return wh + qh + (w > f ? w : f);
}

int gpr_ader_stepper(double *u, const double *ub, const int32_t *nX, int ndim, double dt,
                     const double *dX, int stiff, int flux, const gpr_par *par,
                     const uint8_t *mask, double *scratch, int32_t *status, int nvar,
                     void *stream) {
  if (!u || !ub || !dX || !par || !scratch || !check_grid(nX, ndim))
    return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  long ncb = ndim == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
  long ns = ndim == 1 ? NN : NN * NN;
  double *wh = scratch;
  double *qh = wh + ncb * ns * nvar;
  double *tmp = qh + ncb * NN * ns * nvar;
  int rc = gpr_weno_launcher(wh, ub, nX, ndim, tmp, nvar, stream);
  if (rc)
    return rc;
  rc = gpr_predictor(qh, wh, dt, dX, ndim, nX, stiff, par, mask, status, nvar, stream);
  if (rc)
    return rc;
  return gpr_fv_launcher(u, qh, nX, dt, dX, ndim, 1, 1, flux, par, mask, tmp, nvar, stream);
}

}  // extern "C"

extern "C" {

long gpr_iterate_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!check_grid(nX, ndim))
    return GPR_E_ARG;
  DISPATCH(nvar, O::iterate_scratch(nX, ndim))
}

int gpr_midstepper(double *wh, double dt, const double *dX, int ndim, const int32_t *nX,
                   const gpr_par *par, const uint8_t *mask, int nvar, void *stream) {
  if (!wh || !dX || !par || !check_grid(nX, ndim))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::midstep(wh, dt, nullptr, dX, ndim, nX, P, mask, S(stream)))
}

long gpr_split_scratch_doubles(const int32_t *nX, int ndim, int nvar) {
  if (!check_grid(nX, ndim))
    return GPR_E_ARG;
  DISPATCH(nvar, O::split_scratch(nX, ndim))
}

int gpr_split_stepper(double *u, double *ub, const int32_t *nX, int ndim, double dt,
                      const double *dX, int half_step, int flux, const gpr_par *par,
                      const uint8_t *mask, double *scratch, int nvar, void *stream) {
  if (!u || !ub || !dX || !par || !scratch || !check_grid(nX, ndim))
    return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::split_stepper(u, ub, nX, ndim, dt, nullptr, dX, half_step, flux, P, mask,
                                  scratch, S(stream)))
}

int gpr_iterate_split(double *u, const int32_t *nX, int ndim, const double *dX,
                      const int32_t *bcs, int flux, int half_step, const gpr_par *par,
                      const uint8_t *mask, double *clock, int nsteps, double *scratch,
                      double contorted_tol, int nvar, void *stream) {
  if (!u || !dX || !bcs || !par || !clock || !scratch || nsteps < 0 || !check_grid(nX, ndim))
    return GPR_E_ARG;
  for (int i = 0; i < 2 * ndim; i++)
    if (bcs[i] < 0 || bcs[i] > 5)
      return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::iterate_split(u, nX, ndim, dX, bcs, P, mask, clock, nsteps, scratch,
                                  half_step, flux, S(stream), contorted_tol))
}

int gpr_iterate(double *u, const int32_t *nX, int ndim, const double *dX, const int32_t *bcs,
                int flux, const gpr_par *par, const uint8_t *mask, double *clock, int nsteps,
                double *scratch, int32_t *status, double contorted_tol, int nvar,
                void *stream) {
  if (!u || !dX || !bcs || !par || !clock || !scratch || nsteps < 0 || !check_grid(nX, ndim))
    return GPR_E_ARG;
  for (int i = 0; i < 2 * ndim; i++)
    if (bcs[i] < 0 || bcs[i] > 5)
      return GPR_E_ARG;
  if (int rc = check_flux(flux, ndim))
    return rc;
  DevPar P = make_devpar(*par);
  DISPATCH(nvar, O::iterate(u, nX, ndim, dX, bcs, P, mask, clock, nsteps, scratch, status,
                            S(stream), flux, contorted_tol))
}

int gpr_contorted(const double *u, int64_t ncell, double contorted_tol, int32_t *flag, int nvar,
                  void *stream) {
  if (!u || !flag || ncell < 1)
    return GPR_E_ARG;
  cudaStream_t st = S(stream);
  if (cudaMemsetAsync(flag, 0, sizeof(int32_t), st) != cudaSuccess)
    return GPR_E_CUDA;
  switch (nvar) {
  case 17:
    k_contorted<17><<<blocks(ncell, 256), 256, 0, st>>>(u, ncell, contorted_tol, (int *)flag,
                                                         nullptr);
    break;
  case 14:
    k_contorted<14><<<blocks(ncell, 256), 256, 0, st>>>(u, ncell, contorted_tol, (int *)flag,
                                                         nullptr);
    break;
  case 15:
    k_contorted<15><<<blocks(ncell, 256), 256, 0, st>>>(u, ncell, contorted_tol, (int *)flag,
                                                         nullptr);
    break;
  default:
    return GPR_E_UNSUPPORTED;
  }
  return cuda_rc();
}

int gpr_reset_contorted(double *u, int64_t ncell, double contorted_tol, const gpr_par *pars,
                        int nmat, int32_t *flag, int nvar, void *stream) {
  if (!u || !pars || !flag || ncell < 1 || nmat < 1 || nmat > 2)
    return GPR_E_ARG;
  DevPar P0 = make_devpar(pars[0]), P1 = nmat > 1 ? make_devpar(pars[1]) : P0;
  DISPATCH(nvar, (O::contortion(u, ncell, contorted_tol, P0, P1, (int *)flag, nullptr,
                                S(stream)),
                  cuda_rc()))
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free 1D ADER step.
//
// Some callers cannot allocate device memory at all: a host application
// that owns the whole device through its own fixed pool (and forbids any
// other cudaMalloc), or a latency-critical loop where an allocation would
// synchronise the device.  For them this entry point takes its scratch (the
// WENO reconstruction, the space-time predictor and the face fluxes) from a
// fixed array compiled into the library instead of from the caller.
//
// The array is sized for up to GPR_NOALLOC_MAX_CELLS cells of up to 17
// variables (about 4.5 MB) and every GPU that loads the library holds it
// until the process exits.  Its device address is looked up once per device
// (cudaGetSymbolAddress, with that device current) on the first call made on
// that device, so that first call must come before any stream capture.
// The looked-up address is kept for the life of the process: after a
// cudaDeviceReset (or a release and re-creation of the device's primary
// context) the module may be loaded elsewhere, so the entry point must not be
// used across such a reset.
// Every call shares the array and it keeps the last call's contents; nothing
// in it has to start at zero (each call overwrites what it reads), but calls
// that overlap on the GPU (different streams, or different host threads on
// one device) race on it and must be serialised by the caller.
namespace {

constexpr long kNoallocDoubles =
    ((long)(GPR_NOALLOC_MAX_CELLS + 2) * NN * 17)            // wh
    + ((long)(GPR_NOALLOC_MAX_CELLS + 2) * NN * NN * 17)     // qh
    + ((long)(GPR_NOALLOC_MAX_CELLS + 1) * 2 * 17);          // face fluxes

static __device__ __align__(256) double g_noalloc_scratch[kNoallocDoubles];

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[256] = {nullptr};

int noalloc_scratch(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256)
    return GPR_E_CUDA;
  std::lock_guard<std::mutex> lk(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "gpr_gb300: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return GPR_E_CUDA;
    }
    g_noalloc_ptr[dev] = (double *)p;
  }
  *out = g_noalloc_ptr[dev];
  return GPR_OK;
}

template <class O>
int noalloc_step(double *u, const double *ub, const int32_t *nX, const double *dX, double dt,
                 int stiff, int flux, const DevPar &P, const uint8_t *mask, int32_t *status,
                 double *wh, double *qh, double *fb, cudaStream_t st) {
  int rc;
  if ((rc = O::weno(wh, ub, nX, 1, nullptr, st)))
    return rc;
  if ((rc = O::predictor(qh, wh, dt, nullptr, dX, 1, nX, stiff, P, mask, status, st)))
    return rc;
  // the 1D face pass writes (nx + 1) x 2 x V doubles whatever the flux
  return O::fv(u, qh, nX, dt, nullptr, dX, 1, 1, 1, P, mask, fb, st, flux);
}

}  // namespace

extern "C" int gpr_ader_stepper_1d_noalloc(double *u, const double *ub, int32_t nx, double dt,
                                           double dx, int stiff, int flux, const gpr_par *par,
                                           const uint8_t *mask, int32_t *status, int nvar,
                                           void *stream) {
  if (!u || !ub || !par || nx < 1)
    return GPR_E_ARG;
  if (nx > GPR_NOALLOC_MAX_CELLS || nvar > 17)
    return GPR_E_TOO_LARGE;
  if (flux != GPR_FLUX_RUSANOV && flux != GPR_FLUX_ROE && flux != GPR_FLUX_OSHER)
    return GPR_E_ARG;
  if (nvar != 17 && nvar != 15 && nvar != 14)
    return GPR_E_UNSUPPORTED;
  double *scr = nullptr;
  int rc = noalloc_scratch(&scr);
  if (rc)
    return rc;
  int32_t nX[1] = {nx};
  double dX[1] = {dx};
  long ncb = nx + 2;
  double *wh = scr;
  double *qh = wh + ncb * NN * nvar;
  double *fb = qh + ncb * NN * NN * nvar;
  DevPar P = make_devpar(*par);
  cudaStream_t st = S(stream);
  switch (nvar) {
  case 17:
    return noalloc_step<Ops<L17>>(u, ub, nX, dX, dt, stiff, flux, P, mask, status, wh, qh, fb, st);
  case 15:
    return noalloc_step<Ops15>(u, ub, nX, dX, dt, stiff, flux, P, mask, status, wh, qh, fb, st);
  default:
    return noalloc_step<Ops<L14>>(u, ub, nX, dX, dt, stiff, flux, P, mask, status, wh, qh, fb, st);
  }
}

// ---------------------------------------------------------------------------
// Batched form (many independent 1D instances in one launch per stage).
#include <map>
#include <vector>

namespace {

// Launch shapes chosen for each batch, keyed by the batch's scratch buffer
// (the tables of one batch live there): written by gpr_batch_autotune /
// gpr_batch_set_shapes, reset by gpr_batch_init, read by gpr_batch_iterate
// on the host when it enqueues the launches.
std::mutex g_shapes_mutex;
std::map<const double *, BatchShapes> g_shapes;

BatchShapes shapes_of(const double *scratch) {
  std::lock_guard<std::mutex> lk(g_shapes_mutex);
  auto it = g_shapes.find(scratch);
  return it == g_shapes.end() ? BatchShapes{} : it->second;
}

void shapes_put(const double *scratch, const BatchShapes &sh) {
  std::lock_guard<std::mutex> lk(g_shapes_mutex);
  g_shapes[scratch] = sh;
}

void shapes_drop(const double *scratch) {
  std::lock_guard<std::mutex> lk(g_shapes_mutex);
  g_shapes.erase(scratch);
}

void shapes_to_array(const BatchShapes &sh, int32_t *out) {
  out[0] = sh.weno;
  out[1] = sh.first;
  out[2] = sh.picard;
  out[3] = sh.faces_split;
  out[4] = sh.faces;
  out[5] = sh.cells;
}

bool lane_block(int bs) { return bs == 32 || bs == 64 || bs == 128; }

}  // namespace

extern "C" {

long gpr_batch_scratch_doubles(int ninst, const int32_t *nx, int nvar) {
  if (ninst < 1 || !nx)
    return GPR_E_ARG;
  for (int k = 0; k < ninst; k++)
    if (nx[k] < 2)
      return GPR_E_ARG;
  DISPATCH(nvar, O::batch_layout(ninst, nx).total)
}

int gpr_batch_init(double *clock, int ninst, const int32_t *nx, const double *dx,
                   const int32_t *bcs, const gpr_par *pars, double cfl, double tf,
                   double *scratch, int nvar, void *stream) {
  if (!clock || ninst < 1 || !nx || !dx || !bcs || !pars || !scratch)
    return GPR_E_ARG;
  for (int k = 0; k < ninst; k++)
    if (nx[k] < 2 || !(dx[k] > 0) || bcs[2 * k] < 0 || bcs[2 * k] > 5 || bcs[2 * k + 1] < 0 ||
        bcs[2 * k + 1] > 5)
      return GPR_E_ARG;
  long total = gpr_batch_scratch_doubles(ninst, nx, nvar);
  if (total < 0)
    return (int)total;
  // host images of the tables
  std::vector<DevPar> P(ninst);
  std::vector<int32_t> ou(ninst), oub(ninst), ob(ninst), of(ninst), bc(2 * ninst);
  std::vector<double> idx(ninst), clk(5 * (size_t)ninst);
  long nu = 0, nub = 0, nb = 0, nf = 0;
  for (int k = 0; k < ninst; k++) {
    P[k] = make_devpar(pars[k]);
    ou[k] = (int32_t)nu;
    oub[k] = (int32_t)nub;
    ob[k] = (int32_t)nb;
    of[k] = (int32_t)nf;
    nu += nx[k];
    nub += nx[k] + 2 * NN;
    nb += nx[k] + 2;
    nf += nx[k] + 1;
    bc[2 * k] = bcs[2 * k];
    bc[2 * k + 1] = bcs[2 * k + 1];
    idx[k] = 1.0 / dx[k];
    double *c = clk.data() + 5 * k;
    c[0] = 0.0;
    c[1] = 0.0;
    c[2] = tf;
    c[3] = cfl;
    c[4] = 0.0;
  }
  if (nu >= 0x7fffffff / 4)
    return GPR_E_TOO_LARGE;
  std::vector<int32_t> iu(nu), iub(nub), ib(nb), iff(nf);
  for (int k = 0; k < ninst; k++) {
    for (int c = 0; c < nx[k]; c++)
      iu[ou[k] + c] = k;
    for (int c = 0; c < nx[k] + 2 * NN; c++)
      iub[oub[k] + c] = k;
    for (int c = 0; c < nx[k] + 2; c++)
      ib[ob[k] + c] = k;
    for (int c = 0; c < nx[k] + 1; c++)
      iff[of[k] + c] = k;
  }
  cudaStream_t st = S(stream);
  auto put = [&](long off, const void *src, size_t bytes) {
    return cudaMemcpyAsync(scratch + off, src, bytes, cudaMemcpyHostToDevice, st);
  };
  cudaError_t e = cudaSuccess;
#define PUT(off, vec) \
  if (e == cudaSuccess) e = put(off, vec.data(), vec.size() * sizeof(vec[0]))
  switch (nvar) {
  case 17:
  case 14:
  case 15: {
    BatchLayout lay = batch_layout_v(ninst, nx, nvar);
    PUT(lay.o_par, P);
    PUT(lay.o_iu, iu);
    PUT(lay.o_iub, iub);
    PUT(lay.o_ib, ib);
    PUT(lay.o_if, iff);
    std::vector<int32_t> nxv(nx, nx + ninst);
    PUT(lay.o_nx, nxv);
    PUT(lay.o_ou, ou);
    PUT(lay.o_oub, oub);
    PUT(lay.o_ob, ob);
    PUT(lay.o_of, of);
    PUT(lay.o_bc, bc);
    PUT(lay.o_idx, idx);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(scratch + lay.o_mx, 0, sizeof(unsigned long long) * ninst, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(clock, clk.data(), clk.size() * sizeof(double),
                          cudaMemcpyHostToDevice, st);
    // the host images above must outlive the copies
    if (e == cudaSuccess)
      e = cudaStreamSynchronize(st);
  } break;
  default:
    return GPR_E_UNSUPPORTED;
  }
#undef PUT
  if (e != cudaSuccess) {
    fprintf(stderr, "gpr_gb300: batch init: %s\n", cudaGetErrorString(e));
    return GPR_E_CUDA;
  }
  shapes_drop(scratch);  // new tables: the default shapes until tuned
  return GPR_OK;
}

int gpr_batch_autotune(double *u, double *clock, int ninst, const int32_t *nx, double *scratch,
                       int32_t *shapes, float *times, int nvar, void *stream) {
  if (!u || !clock || ninst < 1 || !nx || !scratch)
    return GPR_E_ARG;
  for (int k = 0; k < ninst; k++)
    if (nx[k] < 2)
      return GPR_E_ARG;
  BatchShapes sh;
  int rc;
  switch (nvar) {
  case 17:
    rc = Ops<L17>::batch_autotune(u, clock, ninst, nx, scratch, sh, times, 3, S(stream));
    break;
  case 14:
    rc = Ops<L14>::batch_autotune(u, clock, ninst, nx, scratch, sh, times, 3, S(stream));
    break;
  case 15:
    rc = Ops15::batch_autotune(u, clock, ninst, nx, scratch, sh, times, 3, S(stream));
    break;
  default:
    return GPR_E_UNSUPPORTED;
  }
  if (rc)
    return rc;
  shapes_put(scratch, sh);
  if (shapes)
    shapes_to_array(sh, shapes);
  return GPR_OK;
}

int gpr_batch_get_shapes(const double *scratch, int32_t *shapes) {
  if (!scratch || !shapes)
    return GPR_E_ARG;
  shapes_to_array(shapes_of(scratch), shapes);
  return GPR_OK;
}

int gpr_batch_set_shapes(const double *scratch, const int32_t *shapes) {
  if (!scratch || !shapes)
    return GPR_E_ARG;
  if (shapes[0] < 32 || shapes[0] > 1024 || shapes[0] % 32 || !lane_block(shapes[1]) ||
      !lane_block(shapes[2]) || (shapes[3] != 0 && shapes[3] != 1) || !lane_block(shapes[4]) ||
      !lane_block(shapes[5]))
    return GPR_E_ARG;
  BatchShapes sh;
  sh.weno = shapes[0];
  sh.first = shapes[1];
  sh.picard = shapes[2];
  sh.faces_split = shapes[3];
  sh.faces = shapes[4];
  sh.cells = shapes[5];
  shapes_put(scratch, sh);
  return GPR_OK;
}

int gpr_batch_iterate(double *u, double *clock, int ninst, const int32_t *nx, int nsteps,
                      double *scratch, int32_t *status, unsigned long long *updates, int nvar,
                      void *stream) {
  if (!u || !clock || ninst < 1 || !nx || nsteps < 0 || !scratch)
    return GPR_E_ARG;
  for (int k = 0; k < ninst; k++)
    if (nx[k] < 2)
      return GPR_E_ARG;
  const BatchShapes sh = shapes_of(scratch);
  DISPATCH(nvar, O::batch_iterate(u, clock, ninst, nx, nsteps, scratch, status, updates,
                                  S(stream), sh))
}

}  // extern "C"
