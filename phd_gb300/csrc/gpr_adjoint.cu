// gpr_adjoint.cu - C ABI of the differentiable 1D step (include/gpr_gb300.h,
// "Adjoint" section): the recorded forward step of the batched form and its
// hand-written backward step (kernels in gpr_adjoint.cuh).
#include <math.h>
#include <stdio.h>

#include "gpr_adjoint.cuh"
#include "gpr_host.cuh"

using namespace gpr;
using namespace gpr::host;

namespace {

// One recorded step: the state entering the step, the converged predictor,
// the state before renormalisation, the step's clock {t, dt, tf, cfl, count}
// per instance, {clipped, argmax cell} per instance, and the argmax scratch.
struct TapeLayout {
  long o_un, o_qh, o_up, o_clk, o_aux, o_amax, o_mcell, total;
};

TapeLayout tape_layout_v(int ninst, const int32_t *nx, int V) {
  BatchLayout b = batch_layout_v(ninst, nx, V);
  Carve cv;
  TapeLayout t;
  t.o_un = cv.take(b.nu * V);
  t.o_qh = cv.take(b.nb * NN * NN * V);
  t.o_up = cv.take(b.nu * V);
  t.o_clk = cv.take(5L * ninst);
  t.o_aux = cv.take(2L * ninst);
  t.o_amax = cv.take((ninst + 1) / 2);
  t.o_mcell = cv.take(b.nu);
  t.total = cv.o;
  return t;
}

// Backward-step scratch: lambda and eigen data at the ends, cotangents of
// qh and wh, stencil cotangents, per-cell material-field and dt partial sums.
struct AdjLayout {
  long o_ev, o_eig, o_qb, o_wb, o_g, o_thf, o_thp, o_dtf, o_dtp, o_mu, o_need, total;
};

AdjLayout adj_layout_v(int ninst, const int32_t *nx, int V) {
  BatchLayout b = batch_layout_v(ninst, nx, V);
  Carve cv;
  AdjLayout a;
  // lambda and eigen data at the cell ends, then at the CFL argmax states
  a.o_ev = cv.take(b.nb * 4 + ninst);
  a.o_eig = cv.take((b.nb * 4 + ninst) * 17);
  a.o_qb = cv.take(b.nb * 4 * V);
  a.o_wb = cv.take(b.nb * 2 * V);
  a.o_g = cv.take(b.nb * V * 3);
  a.o_thf = cv.take(b.nb * 2 * NPD);
  a.o_thp = cv.take(b.nb * NPD);
  a.o_dtf = cv.take(b.nb);
  a.o_dtp = cv.take(b.nb);
  a.o_mu = cv.take(b.nb * 4 * V);
  a.o_need = cv.take((b.nb + 1) / 2);
  a.total = cv.o;
  return a;
}

template <class L> struct Adj {
  static constexpr int V = L::V;
  static constexpr int K = V + NPD;

  static int forward_step(double *u, double *clk, int ninst, const int32_t *nx, double *scr,
                          double *tape, double *dt_io, int dt_mode, double dg_tol, int dg_it,
                          int32_t *status, cudaStream_t st) {
    Consts C = consts();
    C.dg_tol = dg_tol;
    C.dg_it = dg_it;
    C.stiff_tol = fmin(C.stiff_tol, dg_tol);
    C.stiff_it = dg_it > C.stiff_it ? dg_it : C.stiff_it;
    BatchLayout b = batch_layout_v(ninst, nx, V);
    Batch B = batch_view_of(scr, ninst, b, clk);
    double *ub = scr + b.o_ub, *wh = scr + b.o_wh, *qh = scr + b.o_qh, *fb = scr + b.o_fb;
    unsigned long long *mx = (unsigned long long *)(scr + b.o_mx);
    TapeLayout tl = tape_layout_v(ninst, nx, V);
    unsigned int *amax = nullptr;
    double *tclk = nullptr, *aux = nullptr;
    if (tape) {
      amax = (unsigned int *)(tape + tl.o_amax);
      tclk = tape + tl.o_clk;
      aux = tape + tl.o_aux;
      qh = tape + tl.o_qh;
      if (cudaMemcpyAsync(tape + tl.o_un, u, sizeof(double) * b.nu * V,
                          cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
          cudaMemsetAsync(amax, 0xff, sizeof(unsigned int) * ninst, st) != cudaSuccess)
        return GPR_E_CUDA;
    }
    DevPar P0{};
    double *mcell = tape ? tape + tl.o_mcell : nullptr;
    k_b_cfl_max<L><<<blocks(b.nu, 256), 256, 0, st>>>(u, b.nu, mx, B, mcell);
    if (tape)
      k_adj_argmax<<<blocks(b.nu, 256), 256, 0, st>>>(mcell, b.nu, mx, amax, B);
    k_adj_clock_finalize<<<blocks(ninst, 128), 128, 0, st>>>(mx, B, dt_io, dt_mode, tclk, aux,
                                                             amax);
    k_b_boundaries<V><<<blocks(b.nub * V, 256), 256, 0, st>>>(u, ub, b.nub, B);
    k_b_weno<V><<<blocks(b.nb * V, 256), 256, 0, st>>>(wh, ub, b.nb, C, B);
    // every iteration in the Picard kernel (no k_predictor_first): the
    // tightly converged forward the gradients and their finite-difference
    // checks difference keeps one arithmetic path
    k_predictor_picard<L, 1, true><<<blocks(b.nb * NN * NN, 128), 128, 0, st>>>(
        qh, wh, b.nb, nullptr, status, 0.0, nullptr, 1.0, 1.0, 0, P0, C, B, 0);
    int rc = launch_stiff<L, 1, true>(qh, wh, b.nb, nullptr, status, 0.0, nullptr, 1.0, 1.0, P0,
                                      C, st, B);
    if (rc)
      return rc;
    k_faces1d<L, true><<<blocks(b.nf * NN, 128), 128, 0, st>>>(fb, qh, b.nf, nullptr, 0.0,
                                                                nullptr, 1.0, 1, P0, C, B);
    k_cells<L, 1, true><<<blocks(b.nu * NN * NN, 128), 128, 0, st>>>(
        u, qh, fb, nullptr, b.nu, 1, nullptr, 0.0, nullptr, 1.0, 1.0, 1, 1, P0, C, B, FV_BOTH);
    if (tape && cudaMemcpyAsync(tape + tl.o_up, u, sizeof(double) * b.nu * V,
                                cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return GPR_E_CUDA;
    k_b_renorm<V><<<blocks(b.nu, 256), 256, 0, st>>>(u, b.nu, B);
    k_b_clock_advance<<<blocks(ninst, 128), 128, 0, st>>>(B, nullptr);
    return cuda_rc();
  }

  static int backward_step(double *ubar, double *thbar, double *tbar, int frozen, int ninst,
                           const int32_t *nx, const double *scr, const double *tape,
                           double *ascr, int32_t *info, cudaStream_t st) {
    const Consts &C = consts();
    BatchLayout b = batch_layout_v(ninst, nx, V);
    TapeLayout tl = tape_layout_v(ninst, nx, V);
    AdjLayout al = adj_layout_v(ninst, nx, V);
    Batch B = batch_view_of(const_cast<double *>(scr), ninst, b,
                            const_cast<double *>(tape + tl.o_clk));
    const double *un = tape + tl.o_un, *qh = tape + tl.o_qh, *up = tape + tl.o_up,
                 *aux = tape + tl.o_aux;
    double *EV = ascr + al.o_ev, *EIG = ascr + al.o_eig,
           *EVs = EV + b.nb * 4, *EIGs = EIG + b.nb * 4 * Xi<L::THERMAL>::ND,
           *qb = ascr + al.o_qb, *wb = ascr + al.o_wb, *g = ascr + al.o_g,
           *thf = ascr + al.o_thf, *thp = ascr + al.o_thp, *dtf = ascr + al.o_dtf,
           *dtp = ascr + al.o_dtp, *mu = ascr + al.o_mu;
    int32_t *need = (int32_t *)(ascr + al.o_need);
    k_adj_renorm<V><<<blocks(b.nu, 256), 256, 0, st>>>(ubar, up, b.nu, B);
    k_adj_eig<L><<<blocks(b.nb * 4 + ninst, 128), 128, 0, st>>>(qh, b.nb, un, aux, EV, EIG, C,
                                                                  B);
    k_adj_fv<L><<<blocks(b.nb * 2, ADJ_FV_PAIRS), 4 * ADJ_FV_PAIRS, 0, st>>>(
        ubar, qh, EV, EIG, un, up, b.nb, qb, thf, dtf, C, B);
    k_adj_pred_iter<L><<<blocks(b.nb * 4, ADJ_IT_T), ADJ_IT_T, 0, st>>>(qh, qb, b.nb, mu, need,
                                                                         info, C, B);
    // above 48 KB of dynamic shared memory needs the opt-in (per device)
    constexpr size_t dsmem = dense_smem_bytes<V>();
    if (cudaFuncSetAttribute(k_adj_pred_dense<L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)dsmem) != cudaSuccess)
      return GPR_E_CUDA;
    k_adj_pred_dense<L><<<(unsigned)b.nb, 128, dsmem, st>>>(qh, qb, b.nb, need, mu, info, C, B);
    k_adj_pred_post<L><<<blocks(b.nb * 4, 128), 128, 0, st>>>(qh, mu, b.nb, wb, thp, dtp, C, B);
    k_adj_weno<V><<<blocks(b.nb * V, 256), 256, 0, st>>>(wb, un, b.nb, g, C, B);
    k_adj_gather<V><<<blocks(b.nu * V, 256), 256, 0, st>>>(ubar, g, b.nu, B);
    k_adj_reduce<L><<<ninst, 128, 0, st>>>(ubar, thbar, tbar, thf, thp, dtf, dtp, un, aux, EVs,
                                           EIGs, frozen, B);
    return cuda_rc();
  }

  static int point(const double *Q, long count, const DevPar &P, double *JF, double *JS,
                   double *dlam, cudaStream_t st) {
    k_adj_point<L><<<blocks(count * K, 128), 128, 0, st>>>(Q, count, JF, JS, dlam, P);
    return cuda_rc();
  }

  static int point_vjp(const double *Q, long count, const DevPar &P, const double *Fb,
                       const double *Sb, const double *lb, double *qb, double *thb,
                       cudaStream_t st) {
    k_adj_point_vjp<L><<<blocks(count, 128), 128, 0, st>>>(Q, count, Fb, Sb, lb, qb, thb, P);
    return cuda_rc();
  }
};

using L17 = Layout<true, 0>;
using L14 = Layout<false, 0>;

#define ADJ_DISPATCH(nvar, CALL) \
  switch (nvar) {                \
  case 17: {                     \
    using A = Adj<L17>;          \
    return CALL;                 \
  }                              \
  case 14: {                     \
    using A = Adj<L14>;          \
    return CALL;                 \
  }                              \
  default:                       \
    return GPR_E_UNSUPPORTED;    \
  }

bool check_sizes(int ninst, const int32_t *nx) {
  if (ninst < 1 || !nx)
    return false;
  for (int k = 0; k < ninst; k++)
    if (nx[k] < 2)
      return false;
  return true;
}

}  // namespace

extern "C" {

int gpr_adj_num_fields(void) { return NPD; }

int gpr_adj_supported(int ninst, const gpr_par *pars, const int32_t *bcs, int nvar) {
  if (ninst < 1 || !pars || !bcs)
    return GPR_E_ARG;
  if (nvar != 17 && nvar != 14)
    return GPR_E_UNSUPPORTED;
  for (int k = 0; k < ninst; k++) {
    const gpr_par &p = pars[k];
    if (p.EOS != 0 || p.flags != 0 || p.beta != 0.0 || p.Tref != 0.0)
      return GPR_E_UNSUPPORTED;
    for (int s = 0; s < 2; s++)
      if (bcs[2 * k + s] == GPR_BC_MOVING || bcs[2 * k + s] < 0 || bcs[2 * k + s] > 5)
        return GPR_E_UNSUPPORTED;
  }
  return GPR_OK;
}

long gpr_adj_tape_doubles(int ninst, const int32_t *nx, int nvar) {
  if (!check_sizes(ninst, nx))
    return GPR_E_ARG;
  if (nvar != 17 && nvar != 14)
    return GPR_E_UNSUPPORTED;
  return tape_layout_v(ninst, nx, nvar).total;
}

long gpr_adj_scratch_doubles(int ninst, const int32_t *nx, int nvar) {
  if (!check_sizes(ninst, nx))
    return GPR_E_ARG;
  if (nvar != 17 && nvar != 14)
    return GPR_E_UNSUPPORTED;
  return adj_layout_v(ninst, nx, nvar).total;
}

int gpr_adj_forward_step(double *u, double *clock, int ninst, const int32_t *nx,
                         double *scratch, double *tape, double *dt_io, int dt_mode,
                         double dg_tol, int dg_it, int32_t *status, int nvar, void *stream) {
  if (!u || !clock || !scratch || !check_sizes(ninst, nx) || (dt_mode != 0 && dt_mode != 1) ||
      (dt_mode == 1 && !dt_io) || !(dg_tol > 0.0) || dg_it < 1)
    return GPR_E_ARG;
  ADJ_DISPATCH(nvar, A::forward_step(u, clock, ninst, nx, scratch, tape, dt_io, dt_mode, dg_tol,
                                     dg_it, status, S(stream)))
}

int gpr_adj_backward_step(double *ubar, double *thbar, double *tbar, int frozen_dt, int ninst,
                          const int32_t *nx, const double *scratch, const double *tape,
                          double *ascratch, int32_t *info, int nvar, void *stream) {
  if (!ubar || !thbar || !tbar || !scratch || !tape || !ascratch || !info ||
      !check_sizes(ninst, nx))
    return GPR_E_ARG;
  ADJ_DISPATCH(nvar, A::backward_step(ubar, thbar, tbar, frozen_dt, ninst, nx, scratch, tape,
                                      ascratch, info, S(stream)))
}

int gpr_adj_point_jacobians(const double *Q, int64_t count, const gpr_par *par, double *JF,
                            double *JS, double *dlam, int nvar, void *stream) {
  if (!Q || !par || !JF || !JS || !dlam || count < 0)
    return GPR_E_ARG;
  const int32_t bc0[2] = {0, 0};
  if (gpr_adj_supported(1, par, bc0, nvar) != GPR_OK)
    return GPR_E_UNSUPPORTED;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  ADJ_DISPATCH(nvar, A::point(Q, count, P, JF, JS, dlam, S(stream)))
}

int gpr_adj_point_vjp(const double *Q, int64_t count, const gpr_par *par, const double *Fb,
                      const double *Sb, const double *lb, double *qb, double *thb, int nvar,
                      void *stream) {
  if (!Q || !par || !Fb || !Sb || !lb || !qb || !thb || count < 0)
    return GPR_E_ARG;
  const int32_t bc0[2] = {0, 0};
  if (gpr_adj_supported(1, par, bc0, nvar) != GPR_OK)
    return GPR_E_UNSUPPORTED;
  if (count == 0)
    return GPR_OK;
  DevPar P = make_devpar(*par);
  ADJ_DISPATCH(nvar, A::point_vjp(Q, count, P, Fb, Sb, lb, qb, thb, S(stream)))
}

}  // extern "C"
